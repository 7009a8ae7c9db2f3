"""sister_gb300: SiSter's 5-view multiview disparity on GB300 (sm_103a), bit-exact with the reference.

Python mirror of the reference helper class (cpp/include/sister/SisterMultiviewDisparities.hpp:18-119)
over the C ABI of libsister_gb300.so (include/sister_gb300.h):

    m = SisterMultiviewDisparities(center, right, top, left, bottom)   # hpp:22
    multi, horiz, vert = m.compute_disparities(dispCount)               # hpp:26

Inputs are u8 images (h x w gray, or h x w x 3 BGR); outputs are u16 h x w images holding disparity*255.
There is no CPU fallback: if the CUDA library is missing or no GPU is present the calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

__all__ = ["SisterMultiviewDisparities", "Context", "Batch", "Server", "SisterError", "load_library", "LIB_PATH"]

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libsister_gb300.so")

SISTER_OK = 0
SISTER_EINVAL, SISTER_ENOMEM, SISTER_EBUDGET, SISTER_EDEVICE, SISTER_ETIMEOUT, SISTER_ESTATE = -1, -2, -3, -4, -5, -6
SISTER_EBUSY, SISTER_EPENDING = -7, -8
_ERRNAMES = {-1: "EINVAL", -2: "ENOMEM", -3: "EBUDGET", -4: "EDEVICE", -5: "ETIMEOUT", -6: "ESTATE"}

STAGES = {1: "frames", 2: "census", 3: "pair_wta", 5: "masks", 6: "cost", 7: "aggregate", 8: "wta"}
TUNE_SGM_ROWS, TUNE_SGM_CLUSTER, TUNE_SGM_GROUPS, TUNE_SGM_CLUSTERS, TUNE_FULL_DISP, TUNE_WAIT_LIMIT_US = 1, 2, 3, 4, 5, 6
DBG_FRAMES, DBG_CENSUS, DBG_WTA, DBG_MEDIAN, DBG_MASKS, DBG_COST, DBG_SUM0, DBG_DISP, DBG_DP = range(1, 10)


class SisterError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d): %s" % (_ERRNAMES.get(code, "E?"), code, msg))
        self.code = code


_lib = None
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u16p = ctypes.POINTER(ctypes.c_uint16)
_vp = ctypes.c_void_p


class SisterRig(ctypes.Structure):
    """struct sister_rig of include/sister_gb300.h."""
    _fields_ = [("views", ctypes.c_void_p * 5), ("width", ctypes.c_int), ("height", ctypes.c_int),
                ("stride", ctypes.c_int), ("channels", ctypes.c_int), ("max_disparity", ctypes.c_int),
                ("multi", ctypes.c_void_p), ("horiz", ctypes.c_void_p), ("vert", ctypes.c_void_p)]


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load libsister_gb300.so (build it with `python -m sister_gb300.build`). Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError("libsister_gb300.so not built (%s); run `python -m sister_gb300.build`" % p)
    lib = ctypes.CDLL(p)
    lib.sister_ctx_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int]
    lib.sister_ctx_destroy.argtypes = [_vp]
    lib.sister_ctx_destroy.restype = None
    lib.sister_last_error.argtypes = [_vp]
    lib.sister_last_error.restype = ctypes.c_char_p
    lib.sister_load_views.argtypes = [_vp, ctypes.POINTER(_vp), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.sister_load_views_device.argtypes = lib.sister_load_views.argtypes
    lib.sister_set_max_disparity.argtypes = [_vp, ctypes.c_int]
    lib.sister_compute.argtypes = [_vp, _vp, _vp, _vp]
    lib.sister_compute_device.argtypes = [_vp, _vp, _vp, _vp]
    lib.sister_stereo.argtypes = [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp]
    lib.sister_set_stream.argtypes = [_vp, _vp]
    lib.sister_synchronize.argtypes = [_vp]
    lib.sister_device_bytes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.sister_device_bytes.restype = ctypes.c_size_t
    lib.sister_debug_fetch.argtypes = [_vp, ctypes.c_int, ctypes.c_int, _vp, ctypes.c_size_t]
    lib.sister_profile_enable.argtypes = [_vp, ctypes.c_int]
    lib.sister_profile_read.argtypes = [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int), ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_int)]
    lib.sister_tune_set.argtypes = [_vp, ctypes.c_int, ctypes.c_int]
    lib.sister_tune_get.argtypes = [_vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    lib.sister_batch_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_size_t]
    lib.sister_batch_destroy.argtypes = [_vp]
    lib.sister_batch_destroy.restype = None
    lib.sister_batch_last_error.argtypes = [_vp]
    lib.sister_batch_last_error.restype = ctypes.c_char_p
    lib.sister_batch_run.argtypes = [_vp, ctypes.POINTER(SisterRig), ctypes.c_int]
    lib.sister_batch_rig_bytes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.sister_batch_rig_bytes.restype = ctypes.c_size_t
    lib.sister_server_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.c_size_t]
    lib.sister_server_destroy.argtypes = [_vp]
    lib.sister_server_destroy.restype = None
    lib.sister_server_last_error.argtypes = [_vp]
    lib.sister_server_last_error.restype = ctypes.c_char_p
    lib.sister_server_submit.argtypes = [_vp, ctypes.POINTER(SisterRig), ctypes.POINTER(ctypes.c_uint64)]
    lib.sister_server_wait.argtypes = [_vp, ctypes.c_uint64, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    lib.sister_server_stats.argtypes = [_vp, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                        ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int)]
    lib.sister_server_set_limits.argtypes = [_vp, ctypes.c_int, ctypes.c_size_t]
    if path is None:
        _lib = lib
    return lib


def _as_views(views):
    out = []
    for v in views:
        a = np.ascontiguousarray(v, dtype=np.uint8)
        if a.ndim not in (2, 3) or (a.ndim == 3 and a.shape[2] != 3):
            raise ValueError("views must be h x w (gray) or h x w x 3 (BGR) uint8 arrays")
        out.append(a)
    shapes = {a.shape for a in out}
    if len(shapes) != 1:
        raise ValueError("all five views must have the same shape, got %s" % sorted(shapes))
    return out


class Context:
    """One device context (sister_ctx): owns device buffers and a stream; not thread-safe."""

    def __init__(self, device: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.sister_ctx_create(ctypes.byref(h), int(device))
        if rc != SISTER_OK:
            raise SisterError(rc, "sister_ctx_create(device=%d) failed" % device)
        self.h = h
        self.shape = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.sister_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != SISTER_OK:
            raise SisterError(rc, self.lib.sister_last_error(self.h).decode(errors="replace"))

    def load_views(self, views):
        vs = _as_views(views)
        h, w = vs[0].shape[:2]
        ch = 3 if vs[0].ndim == 3 else 1
        arr = (ctypes.c_void_p * 5)(*[v.ctypes.data for v in vs])
        self._check(self.lib.sister_load_views(self.h, arr, w, h, w * ch, ch))
        self.shape = (h, w)
        self._keep = vs

    def load_views_host(self, ptrs, width: int, height: int, stride: int, channels: int = 1):
        """Host pointers (e.g. pinned buffers) in the order center, right, top, left, bottom."""
        arr = (ctypes.c_void_p * 5)(*[int(p) for p in ptrs])
        self._check(self.lib.sister_load_views(self.h, arr, width, height, stride, channels))
        self.shape = (height, width)

    def compute_host(self, multi_ptr=None, horiz_ptr=None, vert_ptr=None):
        """sister_compute into caller-owned host buffers of width*height u16 (blocking)."""
        self._check(self.lib.sister_compute(self.h, multi_ptr, horiz_ptr, vert_ptr))

    def load_views_device(self, ptrs, width: int, height: int, stride: int, channels: int = 1):
        arr = (ctypes.c_void_p * 5)(*[int(p) for p in ptrs])
        self._check(self.lib.sister_load_views_device(self.h, arr, width, height, stride, channels))
        self.shape = (height, width)

    def set_max_disparity(self, dc: int):
        self._check(self.lib.sister_set_max_disparity(self.h, int(dc)))

    def compute(self, multi=True, horiz=False, vert=False):
        if self.shape is None:  # nothing loaded: let the library report the call-order error
            self._check(self.lib.sister_compute(self.h, None, None, None))
        h, w = self.shape
        outs = [np.empty((h, w), np.uint16) if f else None for f in (multi, horiz, vert)]
        ptrs = [o.ctypes.data if o is not None else None for o in outs]
        self._check(self.lib.sister_compute(self.h, *ptrs))
        return outs

    def stereo(self, center, other, dc: int):
        """Two-view doStereo (SisterMultiviewDisparities.hpp:122-150) on one gray image pair: returns (left int16,
        -10 where the LR check rejects; right uint16, the median-filtered right map)."""
        a = np.ascontiguousarray(center, np.uint8)
        b = np.ascontiguousarray(other, np.uint8)
        if a.shape != b.shape or a.ndim != 2:
            raise ValueError("stereo: center and other must be 2-D gray images of the same shape")
        h, w = a.shape
        left = np.empty((h, w), np.int16)
        right = np.empty((h, w), np.uint16)
        self._check(self.lib.sister_stereo(self.h, a.ctypes.data, b.ctypes.data, w, h, w, int(dc), left.ctypes.data,
                                           right.ctypes.data))
        return left, right

    def compute_device(self, multi_ptr=None, horiz_ptr=None, vert_ptr=None):
        self._check(self.lib.sister_compute_device(self.h, multi_ptr, horiz_ptr, vert_ptr))

    def set_stream(self, stream_ptr):
        self._check(self.lib.sister_set_stream(self.h, stream_ptr))

    def synchronize(self):
        self._check(self.lib.sister_synchronize(self.h))

    def profile(self, on: bool = True):
        self._check(self.lib.sister_profile_enable(self.h, int(on)))

    def profile_read(self):
        """[(stage name, ms), ...] of the last compute, in launch order."""
        ms = (ctypes.c_float * 64)()
        st = (ctypes.c_int * 64)()
        n = ctypes.c_int(0)
        self._check(self.lib.sister_profile_read(self.h, ms, st, 64, ctypes.byref(n)))
        return [(STAGES.get(st[k], str(st[k])), float(ms[k])) for k in range(n.value)]

    def tune_set(self, key: int, value: int):
        self._check(self.lib.sister_tune_set(self.h, key, int(value)))

    def tune_get(self, key: int) -> int:
        v = ctypes.c_int(0)
        self._check(self.lib.sister_tune_get(self.h, key, ctypes.byref(v)))
        return v.value

    def plan(self) -> dict:
        return {k: self.tune_get(v) for k, v in (("rows", TUNE_SGM_ROWS), ("cluster", TUNE_SGM_CLUSTER),
                                                  ("groups", TUNE_SGM_GROUPS), ("clusters", TUNE_SGM_CLUSTERS))}

    def debug(self, what: int, index: int, shape, dtype):
        out = np.empty(shape, dtype)
        self._check(self.lib.sister_debug_fetch(self.h, what, index, out.ctypes.data, out.nbytes))
        return out

    def debug_dp(self) -> int:
        v = ctypes.c_int(0)
        self._check(self.lib.sister_debug_fetch(self.h, DBG_DP, 0, ctypes.addressof(v), 4))
        return v.value


class SisterMultiviewDisparities:
    """Drop-in for the reference helper class (SisterMultiviewDisparities.hpp:18-119).

    Views are given in the reference constructor order: center, right, top, left, bottom.
    compute_disparities(dispCount) returns (disp_multiview, disp_horizontal, disp_vertical), u16 h x w
    images of disparity*255, exactly as the reference's output Mats.
    """

    def __init__(self, center, right, top, left, bottom, device: int = 0):
        self.views = _as_views([center, right, top, left, bottom])
        self.ctx = Context(device)
        self.ctx.load_views(self.views)

    def compute_disparities(self, dispCount: int, multiview=True, horizontal=True, vertical=True):
        self.ctx.set_max_disparity(dispCount)
        return tuple(self.ctx.compute(multiview, horizontal, vertical))


class Batch:
    """Batched rigs (sister_batch): run(rigs) computes many rigs at once, bit-identical to Context.compute.

    Each rig is (views, dispCount) or (views, dispCount, (multiview, horizontal, vertical)) with views in the
    reference constructor order; run returns, per rig, the tuple of requested u16 h x w maps (None where a
    mode was not requested)."""

    def __init__(self, device: int = 0, budget_bytes: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.sister_batch_create(ctypes.byref(h), int(device), int(budget_bytes))
        if rc != SISTER_OK:
            raise SisterError(rc, "sister_batch_create(device=%d, budget=%d) failed" % (device, budget_bytes))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.sister_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def rig_bytes(width: int, height: int, dc: int, nmodes: int = 1) -> int:
        return int(load_library().sister_batch_rig_bytes(width, height, dc, nmodes))

    def run(self, rigs):
        arr = (SisterRig * len(rigs))()
        keep, outs = [], []
        for k, rig in enumerate(rigs):
            views, dc = rig[0], rig[1]
            modes = rig[2] if len(rig) > 2 else (True, False, False)
            vs = _as_views(views)
            keep.append(vs)
            h, w = vs[0].shape[:2]
            ch = 1 if vs[0].ndim == 2 else 3
            r = arr[k]
            for v in range(5):
                r.views[v] = vs[v].ctypes.data
            r.width, r.height, r.stride, r.channels, r.max_disparity = w, h, w * ch, ch, int(dc)
            o = tuple(np.empty((h, w), np.uint16) if m else None for m in modes)
            r.multi = o[0].ctypes.data if o[0] is not None else None
            r.horiz = o[1].ctypes.data if o[1] is not None else None
            r.vert = o[2].ctypes.data if o[2] is not None else None
            outs.append(o)
        rc = self.lib.sister_batch_run(self.h, arr, len(rigs))
        if rc != SISTER_OK:
            raise SisterError(rc, self.lib.sister_batch_last_error(self.h).decode(errors="replace"))
        return outs


def _fill_rig(r, views, dc, modes, outputs=None):
    vs = _as_views(views)
    h, w = vs[0].shape[:2]
    ch = 1 if vs[0].ndim == 2 else 3
    for v in range(5):
        r.views[v] = vs[v].ctypes.data
    r.width, r.height, r.stride, r.channels, r.max_disparity = w, h, w * ch, ch, int(dc)
    if outputs is not None:
        it = iter(outputs)
        o = tuple(next(it) if m else None for m in modes)
        for a in o:
            if a is not None and (a.dtype != np.uint16 or a.shape != (h, w) or not a.flags["C_CONTIGUOUS"]):
                raise ValueError("outputs must be C-contiguous uint16 arrays of shape %s" % ((h, w),))
    else:
        o = tuple(np.empty((h, w), np.uint16) if m else None for m in modes)
    r.multi = o[0].ctypes.data if o[0] is not None else None
    r.horiz = o[1].ctypes.data if o[1] is not None else None
    r.vert = o[2].ctypes.data if o[2] is not None else None
    return vs, o


class Server:
    """Serving loop (sister_server): submit(views, dispCount[, modes]) from any thread returns a ticket;
    wait(ticket) returns (outputs, latency_ms). Requests are admitted continuously as stream slots and device
    memory free up, run concurrently on the device, and complete one by one."""

    def __init__(self, device: int = 0, budget_bytes: int = 16 << 30, max_inflight: int | None = None,
                 max_queue: int | None = None):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.sister_server_create(ctypes.byref(h), int(device), int(budget_bytes))
        if rc != SISTER_OK:
            raise SisterError(rc, "sister_server_create(device=%d, budget=%d) failed" % (device, budget_bytes))
        self.h = h
        self._live = {}
        if max_inflight is not None or max_queue is not None:
            self.set_limits(max_inflight or 8, max_queue if max_queue is not None else 1024)

    def set_limits(self, max_inflight: int, max_queue: int):
        rc = self.lib.sister_server_set_limits(self.h, int(max_inflight), ctypes.c_size_t(int(max_queue)))
        if rc != SISTER_OK:
            raise SisterError(rc, "sister_server_set_limits failed")

    def _err(self) -> str:
        return self.lib.sister_server_last_error(self.h).decode(errors="replace")

    def submit(self, views, dc, modes=(True, False, False), outputs=None) -> int:
        """outputs: optional tuple of caller-owned u16 h x w arrays (e.g. in pinned memory) per requested mode."""
        r = SisterRig()
        vs, o = _fill_rig(r, views, dc, modes, outputs)
        t = ctypes.c_uint64(0)
        rc = self.lib.sister_server_submit(self.h, ctypes.byref(r), ctypes.byref(t))
        if rc != SISTER_OK:
            raise SisterError(rc, self._err())
        self._live[t.value] = (vs, o)
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000):
        lat = ctypes.c_double(0)
        rc = self.lib.sister_server_wait(self.h, ticket, int(timeout_ms), ctypes.byref(lat))
        if rc == SISTER_EPENDING:
            raise TimeoutError("request %d still queued or running after %d ms" % (ticket, timeout_ms))
        vs, o = self._live.pop(ticket)
        if rc != SISTER_OK:
            raise SisterError(rc, self._err())
        return o, lat.value

    def stats(self):
        a, c, r = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
        p = ctypes.c_int(0)
        self.lib.sister_server_stats(self.h, ctypes.byref(a), ctypes.byref(c), ctypes.byref(r), ctypes.byref(p))
        return {"admitted": a.value, "completed": c.value, "rejected": r.value, "peak_inflight": p.value}

    def close(self):
        if getattr(self, "h", None):
            self.lib.sister_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
