"""Oracle for the SiSter 5-view disparity path -- TEST INFRASTRUCTURE ONLY.

`port` wraps the portable C restatement (liboracle.so, built from sister_oracle.c on any host).
`ref` wraps the reference's own stage code compiled from its sources (oracle/_ref/libsister_ref.so,
x86 hosts with the reference tree only; see build_ref.sh). Only tests, the smoke check and the CPU
baseline legs of bench.py use this package; the product library never does.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libsister_ref.so")

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u16p = ctypes.POINTER(ctypes.c_uint16)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_f32p = ctypes.POINTER(ctypes.c_float)


def build_port(force: bool = False) -> str:
    """Compile the portable C oracle with OpenMP (gcc, any architecture)."""
    src = os.path.join(HERE, "sister_oracle.c")
    if force or not os.path.exists(PORT_SO) or os.path.getmtime(PORT_SO) < os.path.getmtime(src):
        tmp = PORT_SO + ".tmp.%d" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", src, "-o", tmp])
        os.replace(tmp, PORT_SO)
    return PORT_SO


def reference_tree() -> str | None:
    """The reference project tree named by SISTER_REFERENCE, when it is present and this host can compile its
    SSE4.1 stage code (x86-64); None otherwise."""
    ref = os.environ.get("SISTER_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "cpp", "src", "sister")):
        return None
    return ref if platform.machine().lower() in ("x86_64", "amd64") else None


def reference_available() -> bool:
    """The reference's compiled stage code can be loaded: already built into oracle/_ref (on an x86-64 host), or
    buildable from the tree named by SISTER_REFERENCE."""
    if platform.machine().lower() not in ("x86_64", "amd64"):
        return False
    return os.path.exists(REF_SO) or reference_tree() is not None


def build_ref(force: bool = False, tree: str | None = None) -> str | None:
    """Compile the reference's stage sources + glue from `tree` (default: SISTER_REFERENCE) into oracle/_ref;
    returns the library path, or None when it cannot be built or loaded here."""
    if tree:
        os.environ["SISTER_REFERENCE"] = tree
    src = reference_tree()
    if src and (force or not os.path.exists(REF_SO)):
        subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), src], stdout=subprocess.DEVNULL)
    return REF_SO if reference_available() and os.path.exists(REF_SO) else None


def _ptr(a: np.ndarray, t):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(t)


class _Lib:
    def __init__(self, path: str):
        self.lib = ctypes.CDLL(path)


class Port(_Lib):
    """The portable C oracle (sister_oracle.h)."""

    def __init__(self, path: str | None = None):
        super().__init__(path or build_port())
        L = self.lib
        L.orc_compute.restype = ctypes.c_int
        L.orc_compute_stream.restype = ctypes.c_int
        L.orc_num_threads.restype = ctypes.c_int

    @staticmethod
    def _views(views):
        vs = [np.ascontiguousarray(v, dtype=np.uint8) for v in views]
        arr = (_u8p * 5)(*[_ptr(v, _u8p) for v in vs])
        return vs, arr

    def num_threads(self) -> int:
        return int(self.lib.orc_num_threads())

    def frames(self, views, dc):
        h, w = views[0].shape
        Wp, Hp = w + 2 * dc, h + 2 * dc
        vs, arr = self._views(views)
        out = np.zeros(8 * Wp * Hp, np.uint8)
        self.lib.orc_frames(arr, w, h, dc, _ptr(out, _u8p))
        res = []
        for k in range(8):
            f = k // 2
            rows, cols = (Wp, Hp) if f & 1 else (Hp, Wp)
            res.append(out[k * Wp * Hp:(k + 1) * Wp * Hp].reshape(rows, cols))
        return res

    def census(self, img):
        img = np.ascontiguousarray(img, np.uint8)
        H, W = img.shape
        out = np.zeros((H, W), np.uint64)
        self.lib.orc_census(_ptr(img, _u8p), W, H, _ptr(out, _u64p))
        return out

    def cost_volume(self, cc, cn, D):
        H, W = cc.shape
        vol = np.zeros((H, W, D), np.uint16)
        self.lib.orc_cost_volume(_ptr(cc, _u64p), _ptr(cn, _u64p), W, H, D, _ptr(vol, _u16p))
        return vol

    def wta_lr(self, cc, cn, D):
        H, W = cc.shape
        L = np.zeros((H, W), np.uint16)
        R = np.zeros((H, W), np.uint16)
        self.lib.orc_wta_lr(_ptr(cc, _u64p), _ptr(cn, _u64p), W, H, D, _ptr(L, _u16p), _ptr(R, _u16p))
        return L, R

    def median_inplace(self, a):
        a = np.ascontiguousarray(a, np.uint16).copy()
        H, W = a.shape
        self.lib.orc_median_inplace(_ptr(a, _u16p), W, H)
        return a

    def lrc_mask(self, L, R, dc):
        H, W = L.shape
        m = np.zeros((H, W), np.uint8)
        self.lib.orc_lrc_mask(_ptr(L, _u16p), _ptr(R, _u16p), W, H, dc, _ptr(m, _u8p))
        return m

    def sgm(self, C, npasses: int = 2):
        C = np.ascontiguousarray(C, np.uint16)
        H, W, D = C.shape
        S = np.zeros_like(C)
        self.lib.orc_sgm_passes(_ptr(C, _u16p), W, H, D, _ptr(S, _u16p), int(npasses))
        return S

    def masked_cost(self, census, masks, dc, mode):
        """census: 8 frame census images (u64), masks: 4 x Hp x Wp (u8) -> M (Hp x Wp x dc u16)."""
        cs = [np.ascontiguousarray(c, np.uint64) for c in census]
        ms = [np.ascontiguousarray(m, np.uint8) for m in masks]
        Hp, Wp = ms[0].shape
        carr = (_u64p * 8)(*[_ptr(c, _u64p) for c in cs])
        marr = (_u8p * 4)(*[_ptr(m, _u8p) for m in ms])
        M = np.zeros((Hp, Wp, dc), np.uint16)
        self.lib.orc_masked_cost(carr, marr, Wp, Hp, dc, int(mode), _ptr(M, _u16p))
        return M

    def wta_right_vol(self, vol):
        vol = np.ascontiguousarray(vol, np.uint16)
        H, W, D = vol.shape
        out = np.zeros((H, W), np.uint16)
        self.lib.orc_wta_right_vol(_ptr(vol, _u16p), W, H, D, _ptr(out, _u16p))
        return out

    def lrcheck(self, L, R):
        L = np.ascontiguousarray(L, np.uint16)
        R = np.ascontiguousarray(R, np.uint16)
        H, W = L.shape
        out = np.zeros((H, W), np.int16)
        self.lib.orc_lrcheck(_ptr(L, _u16p), _ptr(R, _u16p), W, H, _ptr(out, ctypes.POINTER(ctypes.c_int16)))
        return out

    def stereo(self, center, other, D):
        """doStereo: (L with -10 where the LR check rejects, median-filtered R)."""
        a = np.ascontiguousarray(center, np.uint8)
        b = np.ascontiguousarray(other, np.uint8)
        h, w = a.shape
        L = np.zeros((h, w), np.int16)
        R = np.zeros((h, w), np.uint16)
        rc = self.lib.orc_stereo(_ptr(a, _u8p), _ptr(b, _u8p), w, h, D, _ptr(L, ctypes.POINTER(ctypes.c_int16)),
                                 _ptr(R, _u16p))
        if rc:
            raise MemoryError("oracle stereo: out of memory")
        return L, R

    def wta_left_vol(self, vol):
        vol = np.ascontiguousarray(vol, np.uint16)
        H, W, D = vol.shape
        disp = np.zeros((H, W), np.uint16)
        self.lib.orc_wta_left_vol(_ptr(vol, _u16p), W, H, D, _ptr(disp, _u16p))
        return disp

    def compute(self, views, dc, modes=(True, True, True), masks=False):
        """compute_disparities: returns (multi, horiz, vert[, masks]); skipped modes are None."""
        h, w = views[0].shape
        vs, arr = self._views(views)
        outs = [np.zeros((h, w), np.uint16) if m else None for m in modes]
        mk = np.zeros((4, h + 2 * dc, w + 2 * dc), np.uint8) if masks else None
        ptrs = [_ptr(o, _u16p) if o is not None else None for o in outs]
        rc = self.lib.orc_compute(arr, w, h, dc, ptrs[0], ptrs[1], ptrs[2], _ptr(mk, _u8p) if mk is not None else None)
        if rc != 0:
            raise RuntimeError("orc_compute failed with %d" % rc)
        return (*outs, mk) if masks else tuple(outs)

    def compute_stream(self, views, dc, mode: int = 0, padded: bool = False):
        """One mode of compute_disparities in bounded memory (orc_compute_stream): returns the w x h output,
        or (output, padded disparity map) with padded=True."""
        h, w = views[0].shape
        vs, arr = self._views(views)
        out = np.zeros((h, w), np.uint16)
        pad = np.zeros((h + 2 * dc, w + 2 * dc), np.uint16) if padded else None
        rc = self.lib.orc_compute_stream(arr, w, h, dc, int(mode), _ptr(out, _u16p),
                                         _ptr(pad, _u16p) if pad is not None else None)
        if rc != 0:
            raise RuntimeError("orc_compute_stream failed with %d" % rc)
        return (out, pad) if padded else out


class Ref(_Lib):
    """The reference's own stage code (census.cpp, postprocess.cpp, sgm.cpp) + restated OpenCV glue."""

    def __init__(self, path: str | None = None):
        p = path or build_ref()
        if p is None:
            raise RuntimeError("reference build unavailable on this host")
        super().__init__(p)
        self.lib.ref_compute.restype = ctypes.c_int

    def census(self, img):
        img = np.ascontiguousarray(img, np.uint8)
        H, W = img.shape
        out = np.zeros((H, W), np.uint64)
        self.lib.ref_census(_ptr(img, _u8p), W, H, _ptr(out, _u64p))
        return out

    def ad_census(self, a, b, D):
        a = np.ascontiguousarray(a, np.uint8)
        b = np.ascontiguousarray(b, np.uint8)
        H, W = a.shape
        vol = np.zeros((H, W, D), np.uint16)
        self.lib.ref_ad_census(_ptr(a, _u8p), _ptr(b, _u8p), W, H, D, _ptr(vol, _u16p))
        return vol

    def wta(self, vol, right: bool):
        vol = np.ascontiguousarray(vol, np.uint16)
        H, W, D = vol.shape
        out = np.zeros((H, W), np.float32)
        self.lib.ref_wta(_ptr(vol, _u16p), W, H, D, int(right), _ptr(out, _f32p))
        return out

    def median_inplace(self, a):
        a = np.ascontiguousarray(a, np.float32).copy()
        H, W = a.shape
        self.lib.ref_median_inplace(_ptr(a, _f32p), W, H)
        return a

    def lrcheck(self, L, R):
        L = np.ascontiguousarray(L, np.float32).copy()
        R = np.ascontiguousarray(R, np.float32)
        H, W = L.shape
        self.lib.ref_lrcheck(_ptr(L, _f32p), _ptr(R, _f32p), W, H)
        return L

    def sgm(self, C):
        C = np.ascontiguousarray(C, np.uint16)
        H, W, D = C.shape
        S = np.zeros_like(C)
        self.lib.ref_sgm(_ptr(C, _u16p), W, H, D, _ptr(S, _u16p))
        return S

    def stereo(self, center, other, D):
        """doStereo (hpp:122-150) from the reference's own stages: ad_census, sgm, WTALeft / WTARight, in-place
        medians, doLRCheck. Returns (L as float32 with -10 where rejected, R as float32)."""
        S = self.sgm(self.ad_census(center, other, D))
        L = self.median_inplace(self.wta(S, right=False))
        R = self.median_inplace(self.wta(S, right=True))
        return self.lrcheck(L, R), R

    def compute(self, views, dc, modes=(True, True, True)):
        h, w = views[0].shape
        vs = [np.ascontiguousarray(v, np.uint8) for v in views]
        arr = (_u8p * 5)(*[_ptr(v, _u8p) for v in vs])
        outs = [np.zeros((h, w), np.uint16) if m else None for m in modes]
        ptrs = [_ptr(o, _u16p) if o is not None else None for o in outs]
        rc = self.lib.ref_compute(arr, w, h, dc, ptrs[0], ptrs[1], ptrs[2])
        if rc != 0:
            raise RuntimeError("ref_compute failed with %d" % rc)
        return tuple(outs)
