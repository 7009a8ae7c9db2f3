"""GPU parity: the CUDA path through the C ABI against the oracle (stage by stage) and against the golden
fixtures made by the reference's own compiled code. Integer work, so every comparison is bit-exact."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_small, out_sha, small_golden_files, views_sha

import sister_gb300 as sg
from sister_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    c = sg.Context(0)
    c.tune_set(sg.TUNE_FULL_DISP, 1)  # keep the padded winner-take-all map for the stage checks
    yield c
    c.close()


def _stage_check(ctx, port, views, dc, modes=(True, True, True)):
    """Run the GPU pipeline and compare every intermediate with the oracle."""
    h, w = views[0].shape
    Wp, Hp = w + 2 * dc, h + 2 * dc
    ctx.load_views(views)
    ctx.set_max_disparity(dc)
    outs = ctx.compute(*modes)
    frames = port.frames(views, dc)
    census = []
    for k in range(8):
        fr = ctx.debug(sg.DBG_FRAMES, k, frames[k].shape, np.uint8)
        assert np.array_equal(fr, frames[k]), "frame %d" % k
        cs = ctx.debug(sg.DBG_CENSUS, k, frames[k].shape, np.uint64)
        ce = port.census(frames[k])
        assert np.array_equal(cs, ce), "census %d: %d px" % (k, int((cs != ce).sum()))
        census.append(ce)
    masks = []
    for f in range(4):
        L, R = port.wta_lr(census[2 * f], census[2 * f + 1], dc)
        shp = census[2 * f].shape
        gl = ctx.debug(sg.DBG_WTA, 2 * f, shp, np.uint16)
        gr = ctx.debug(sg.DBG_WTA, 2 * f + 1, shp, np.uint16)
        assert np.array_equal(gl, L), "wta-left frame %d: %d px" % (f, int((gl != L).sum()))
        assert np.array_equal(gr, R), "wta-right frame %d: %d px" % (f, int((gr != R).sum()))
        Lm, Rm = port.median_inplace(L), port.median_inplace(R)
        ml = ctx.debug(sg.DBG_MEDIAN, 2 * f, shp, np.uint16)
        mr = ctx.debug(sg.DBG_MEDIAN, 2 * f + 1, shp, np.uint16)
        assert np.array_equal(ml, Lm), "median-left frame %d: %d px" % (f, int((ml != Lm).sum()))
        assert np.array_equal(mr, Rm), "median-right frame %d: %d px" % (f, int((mr != Rm).sum()))
        mf = port.lrc_mask(Lm, Rm, dc)
        gm = ctx.debug(sg.DBG_MASKS, f, (Hp, Wp), np.uint8)
        if f == 0:
            mo = mf
        elif f == 2:
            mo = mf[:, ::-1]
        elif f == 1:
            mo = mf[::-1, ::-1].T
        else:
            mo = mf[::-1, :].T
        assert np.array_equal(gm, mo), "mask frame %d: %d px" % (f, int((gm != mo).sum()))
        masks.append(np.ascontiguousarray(mo))
    last = max(m for m in range(3) if modes[m])
    dp = ctx.debug_dp()
    M = port.masked_cost(census, masks, dc, last)
    gM = ctx.debug(sg.DBG_COST, 0, (Hp, Wp, dp), np.uint16)
    assert np.array_equal(gM[:, :, :dc], M), "cost: %d cells" % int((gM[:, :, :dc] != M).sum())
    assert (gM[:, :, dc:] == 0x7FFF).all()
    S0 = port.sgm(M, npasses=1)
    gS0 = ctx.debug(sg.DBG_SUM0, 0, (Hp, Wp, dp), np.uint16)
    bad = gS0[:, :, :dc] != S0
    assert not bad.any(), "pass-0 sum: %d cells, first at %s" % (int(bad.sum()), np.argwhere(bad)[:3].tolist())
    S = port.sgm(M)
    disp = port.wta_left_vol(S)
    gd = ctx.debug(sg.DBG_DISP, last, (Hp, Wp), np.uint16)
    assert np.array_equal(gd, disp), "disparity: %d px" % int((gd != disp).sum())
    want = port.compute(views, dc, modes=modes)
    for m in range(3):
        if modes[m]:
            assert np.array_equal(outs[m], want[m]), "mode %d output" % m


@pytest.mark.parametrize("w,h,dc,seed", [(64, 48, 16, 1), (96, 64, 24, 2), (128, 96, 40, 3), (160, 120, 64, 4)])
def test_stages_synthetic(ctx, port, w, h, dc, seed):
    views, _ = synth.make_rig(w, h, 2, max(dc - 8, 4), seed=seed, tiles=4)
    _stage_check(ctx, port, views, dc)


@pytest.mark.parametrize("w,h,dc", [(24, 16, 8), (40, 32, 16), (36, 60, 96), (32, 20, 200), (16, 12, 264)])
def test_stages_random(ctx, port, w, h, dc):
    rng = np.random.default_rng(w * h + dc)
    views = [rng.integers(0, 256, (h, w), dtype=np.uint8) for _ in range(5)]
    _stage_check(ctx, port, views, dc, modes=(True, False, False))


@pytest.mark.parametrize("path", small_golden_files(), ids=os.path.basename)
def test_golden_small(ctx, path):
    views, dc, gold, sha = load_small(path)
    assert views_sha(views) == sha
    ctx.load_views(views)
    ctx.set_max_disparity(dc)
    got = ctx.compute(True, True, True)
    for k in range(3):
        assert np.array_equal(got[k], gold[k]), "mode %d: %d px" % (k, int((got[k] != gold[k]).sum()))


def test_golden_c1(ctx):
    z = np.load(os.path.join(GOLDEN, "c1_640x480_dc192.npz"))
    (views, _), dc = synth.rig_c1(int(z["seed"]))
    assert views_sha(views) == str(z["views_sha"])
    m = sg.SisterMultiviewDisparities(*views)
    multi, horiz, vert = m.compute_disparities(dc)
    assert out_sha(multi) == str(z["multi_sha"]), "%d px differ" % int(((multi // 255) != z["multi_d"]).sum())
    assert out_sha(horiz) == str(z["horiz_sha"])
    assert out_sha(vert) == str(z["vert_sha"])


def test_golden_c2(ctx):
    z = np.load(os.path.join(GOLDEN, "c2_1920x1080_dc256.npz"))
    (views, _), dc = synth.rig_c2(int(z["seed"]))
    assert views_sha(views) == str(z["views_sha"])
    ctx.load_views(views)
    ctx.set_max_disparity(dc)
    multi, horiz, vert = ctx.compute(True, True, True)
    assert out_sha(multi) == str(z["multi_sha"]), "%d px differ" % int(((multi // 255) != z["multi_d"]).sum())
    assert out_sha(horiz) == str(z["horiz_sha"])
    assert out_sha(vert) == str(z["vert_sha"])


def test_max_disparity_512(ctx, port):
    """dc = 512 (stress-rig disparity range, beyond the reference's WTARight limit) vs the oracle."""
    rng = np.random.default_rng(512)
    views = [rng.integers(0, 256, (8, 16), dtype=np.uint8) for _ in range(5)]
    ctx.load_views(views)
    ctx.set_max_disparity(512)
    got = ctx.compute(True, False, False)[0]
    want = port.compute(views, 512, modes=(True, False, False))[0]
    assert np.array_equal(got, want)


def test_max_disparity_512_band_heights(gpu_lib, port):
    """dc = 512 with bands of 9 rows (cost copies of 4 pixels) and of 11 and 12 rows (copies of 2 pixels, the
    aggregation's second instantiation at this d-stride) vs the oracle."""
    rng = np.random.default_rng(1512)
    views = [rng.integers(0, 256, (12, 20), dtype=np.uint8) for _ in range(5)]
    want = port.compute(views, 512, modes=(True, False, False))[0]
    for rows in (9, 11, 12):
        c = sg.Context(0)
        c.tune_set(sg.TUNE_SGM_ROWS, rows)
        c.load_views(views)
        c.set_max_disparity(512)
        got = c.compute(True, False, False)[0]
        assert c.plan()["rows"] == rows
        assert np.array_equal(got, want), "%d-row bands: %d px differ" % (rows, int((got != want).sum()))
        c.close()


def test_bgr_input_matches_gray(ctx):
    views, _ = synth.make_rig(96, 64, 2, 16, seed=9, tiles=3)
    ctx.load_views(views)
    ctx.set_max_disparity(24)
    gray = ctx.compute(True, False, False)[0]
    bgr = [np.repeat(v[:, :, None], 3, axis=2) for v in views]
    ctx.load_views(bgr)
    assert np.array_equal(ctx.compute(True, False, False)[0], gray)
    # a colour image goes through the fixed-point BGR2GRAY weights
    rng = np.random.default_rng(3)
    col = [rng.integers(0, 256, (64, 96, 3), dtype=np.uint8) for _ in range(5)]
    conv = []
    for c in col:
        b, g, r = (c[:, :, k].astype(np.uint32) for k in range(3))
        conv.append(((b * 1868 + g * 9617 + r * 4899 + 8192) >> 14).astype(np.uint8))
    ctx.load_views(col)
    a = ctx.compute(True, False, False)[0]
    ctx.load_views(conv)
    assert np.array_equal(ctx.compute(True, False, False)[0], a)


def test_repeat_and_regeometry(ctx, port):
    """Buffers are reused across calls and geometries; results do not depend on call history."""
    a, _ = synth.make_rig(128, 96, 2, 30, seed=21, tiles=3)
    b, _ = synth.make_rig(64, 48, 2, 12, seed=22, tiles=3)
    res = []
    for views, dc in ((a, 40), (b, 16), (a, 40), (a, 40)):
        ctx.load_views(views)
        ctx.set_max_disparity(dc)
        res.append(ctx.compute(True, False, False)[0])
    assert np.array_equal(res[0], res[2]) and np.array_equal(res[2], res[3])
    assert np.array_equal(res[1], port.compute(b, 16, modes=(True, False, False))[0])


def test_errors(ctx):
    c = sg.Context(0)
    with pytest.raises(sg.SisterError) as e:
        c.compute(True, False, False)
    assert e.value.code == -6
    with pytest.raises(sg.SisterError) as e:
        c.set_max_disparity(12)
    assert e.value.code == -1
    with pytest.raises(sg.SisterError) as e:
        c.load_views([np.zeros((30, 40), np.uint8)] * 5)
    assert e.value.code == -1
    c.close()


def test_full_disp_switch(gpu_lib):
    """The padded map is only kept on request; the outputs are the same either way."""
    views, _ = synth.make_rig(96, 64, 2, 20, seed=9, tiles=4)
    c = sg.Context(0)
    c.load_views(views)
    c.set_max_disparity(24)
    crop_only = c.compute(True, True, True)
    with pytest.raises(sg.SisterError):
        c.debug(sg.DBG_DISP, 0, (64 + 48, 96 + 48), np.uint16)
    c.tune_set(sg.TUNE_FULL_DISP, 1)
    full = c.compute(True, True, True)
    disp = c.debug(sg.DBG_DISP, 0, (64 + 48, 96 + 48), np.uint16)
    c.close()
    for a, b in zip(crop_only, full):
        assert np.array_equal(a, b)
    assert np.array_equal(full[0].astype(np.int64), np.minimum(disp[24:88, 24:120].astype(np.int64) * 255, 65535))
