"""sister_aggregate_static: the allocation-free aggregation entry point, for callers that cannot allocate
device memory when they need a result (fixed-budget robot / ROS callbacks, code inside a framework that
owns all device allocations). Checked through the C ABI against sister_compute on the same rig, twice in
a row (the static scratch arena is shared and keeps the previous call's contents)."""
import ctypes

import numpy as np
import pytest

import sister_gb300 as sg
from sister_gb300 import synth

pytestmark = pytest.mark.gpu


def _entry(lib):
    f = lib.sister_aggregate_static
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]
    f.restype = ctypes.c_int
    return f


def test_static_entry_matches_compute(gpu_lib):
    import torch

    w, h, dc = 128, 96, 40
    views, _ = synth.make_rig(w, h, 2, 32, seed=31, tiles=4)
    ctx = sg.Context(0)
    ctx.tune_set(sg.TUNE_FULL_DISP, 1)
    ctx.load_views(views)
    ctx.set_max_disparity(dc)
    multi = ctx.compute(True, False, False)[0]           # existing entry point
    Wp, Hp = w + 2 * dc, h + 2 * dc
    dp = ctx.debug_dp()
    cost = ctx.debug(sg.DBG_COST, 0, (Hp, Wp, dp), np.uint16)  # its masked cost volume (mode 0)
    disp = ctx.debug(sg.DBG_DISP, 0, (Hp, Wp), np.uint16)
    ctx.close()

    f = _entry(gpu_lib)
    d_cost = torch.from_numpy(cost.view(np.int16)).cuda()
    d_out = torch.empty((h, w), dtype=torch.int16, device="cuda")
    d_disp = torch.empty((Hp, Wp), dtype=torch.int16, device="cuda")
    err = ctypes.create_string_buffer(256)
    for call in range(2):
        d_out.fill_(-1)
        d_disp.fill_(-1)
        torch.cuda.synchronize()
        rc = f(d_cost.data_ptr(), w, h, dc, dp, d_out.data_ptr(), d_disp.data_ptr(), None, err, 256)
        assert rc == 0, (call, rc, err.value)
        got = d_out.cpu().numpy().view(np.uint16)
        assert np.array_equal(got, multi), "call %d: %d px differ" % (call, int((got != multi).sum()))
        assert np.array_equal(d_disp.cpu().numpy().view(np.uint16), disp), "call %d: padded disparity" % call


def test_static_entry_rejects_oversized_and_bad_layout(gpu_lib):
    import torch

    f = _entry(gpu_lib)
    err = ctypes.create_string_buffer(256)
    d = torch.empty(16, dtype=torch.int16, device="cuda")
    # 1920x1080 at dc 256 needs ~2 GB of scratch: beyond the arena -> SISTER_EBUDGET with the sizes
    rc = f(d.data_ptr(), 1920, 1080, 256, 256, None, None, None, err, 256)
    assert rc == -3 and b"static arena" in err.value
    rc = f(d.data_ptr(), 128, 96, 40, 32, None, None, None, err, 256)  # wrong d-stride for dc 40
    assert rc == -1 and b"d-stride" in err.value
    rc = f(None, 128, 96, 40, 64, None, None, None, err, 256)
    assert rc == -1
