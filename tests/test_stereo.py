"""Two-view doStereo (SisterMultiviewDisparities.hpp:122-150): the oracle against fixtures made by the reference's own
compiled stages (ad_census, sgm, WTALeft / WTARight, in-place medians, doLRCheck) and, on the GPU, the library's
sister_stereo against both. Integer disparities and the reference's -10 marker, so every comparison is bit-exact."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

import oracle
from sister_gb300 import synth

STEREO_FILES = sorted(glob.glob(os.path.join(GOLDEN, "stereo_*.npz")))
needs_ref = pytest.mark.skipif(not oracle.reference_available(), reason="reference tree not present on this host")


def _load(path):
    z = np.load(path)
    return z["center"], z["other"], int(z["dc"]), z["left"], z["right"]


def test_stereo_fixtures_exist():
    assert len(STEREO_FILES) >= 5


@pytest.mark.parametrize("path", STEREO_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_port_stereo_matches_golden(port, path):
    center, other, dc, left, right = _load(path)
    L, R = port.stereo(center, other, dc)
    assert np.array_equal(L, left) and np.array_equal(R, right)


def test_golden_stereo_has_rejections():
    # the LR check must be exercised: some pixels of the synthetic pairs are rejected (-10), most are kept
    _, _, _, left, _ = _load(os.path.join(GOLDEN, "stereo_synth_160x120_dc48.npz"))
    frac = float((left == -10).mean())
    assert 0.005 < frac < 0.5


@needs_ref
@pytest.mark.parametrize("H,W,D", [(20, 24, 8), (36, 64, 24), (48, 40, 40)])
def test_port_stereo_vs_ref(port, H, W, D):
    ref = oracle.Ref()
    rng = np.random.default_rng(H * W + D)
    a = rng.integers(0, 256, (H, W), dtype=np.uint8)
    b = np.roll(a, -D // 3, axis=1) if W > D else rng.integers(0, 256, (H, W), dtype=np.uint8)
    L, R = port.stereo(a, b, D)
    Lr, Rr = ref.stereo(a, b, D)
    assert np.array_equal(L.astype(np.float32), Lr) and np.array_equal(R.astype(np.float32), Rr)


@pytest.fixture(scope="module")
def ctx(gpu_lib):
    import sister_gb300 as sg

    c = sg.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", STEREO_FILES, ids=lambda p: os.path.basename(p)[:-4])
def test_gpu_stereo_matches_golden(ctx, path):
    center, other, dc, left, right = _load(path)
    L, R = ctx.stereo(center, other, dc)
    assert np.array_equal(L, left) and np.array_equal(R, right)


@pytest.mark.gpu
@pytest.mark.parametrize("w,h,dc", [(64, 48, 8), (128, 96, 40), (256, 64, 200), (96, 80, 264), (544, 36, 512)])
def test_gpu_stereo_matches_oracle(ctx, port, w, h, dc):
    # every disparity-stride class, including dc > 256 where the reference's WTARight overflows its stack buffer
    # and the restated argmin is the contract
    views, _ = synth.make_rig(w, h, 2, max(6, min(dc - 8, w // 3)), seed=w + h + dc, tiles=4)
    L, R = ctx.stereo(views[0], views[1], dc)
    Lo, Ro = port.stereo(views[0], views[1], dc)
    assert np.array_equal(L, Lo) and np.array_equal(R, Ro)


@pytest.mark.gpu
def test_gpu_stereo_then_multiview(ctx, port):
    # a stereo call between multiview computes leaves the multiview results intact
    views, _ = synth.make_rig(96, 64, 2, 20, seed=5, tiles=4)
    ctx.load_views(views)
    ctx.set_max_disparity(24)
    first = ctx.compute(True, False, False)[0]
    ctx.stereo(views[0], views[3], 16)
    again = ctx.compute(True, False, False)[0]
    assert np.array_equal(first, again)


@pytest.mark.gpu
def test_gpu_stereo_errors(ctx):
    import sister_gb300 as sg

    a = np.zeros((30, 40), np.uint8)
    with pytest.raises(sg.SisterError):
        ctx.stereo(a, a, 16)  # height not a multiple of 4
    b = np.zeros((32, 40), np.uint8)
    with pytest.raises(sg.SisterError):
        ctx.stereo(b, b, 12)  # dc not a multiple of 8
