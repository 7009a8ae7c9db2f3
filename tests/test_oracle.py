"""CPU tests of the oracle: against the golden fixtures (made by the reference's own compiled code) and,
where the reference tree and an x86 host are available, stage by stage against that compiled code."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_small, out_sha, small_golden_files, views_sha

import oracle
from sister_gb300 import synth


@pytest.mark.parametrize("path", small_golden_files(), ids=os.path.basename)
def test_port_matches_golden_small(port, path):
    views, dc, gold, sha = load_small(path)
    assert views_sha(views) == sha
    got = port.compute(views, dc)
    for k, name in enumerate(("multi", "horiz", "vert")):
        assert np.array_equal(got[k], gold[k]), "%s differs in %d px" % (name, int((got[k] != gold[k]).sum()))


def test_generator_reproduces_c1_inputs():
    z = np.load(os.path.join(GOLDEN, "c1_640x480_dc192.npz"))
    (views, _), dc = synth.rig_c1(int(z["seed"]))
    assert dc == int(z["dc"])
    assert views_sha(views) == str(z["views_sha"])


def test_generator_reproduces_c2_inputs():
    z = np.load(os.path.join(GOLDEN, "c2_1920x1080_dc256.npz"))
    (views, _), dc = synth.rig_c2(int(z["seed"]))
    assert dc == int(z["dc"])
    assert views_sha(views) == str(z["views_sha"])


@pytest.mark.slow
def test_port_matches_golden_c1(port):
    z = np.load(os.path.join(GOLDEN, "c1_640x480_dc192.npz"))
    (views, _), dc = synth.rig_c1(int(z["seed"]))
    multi, horiz, vert = port.compute(views, dc)
    assert out_sha(multi) == str(z["multi_sha"])
    assert out_sha(horiz) == str(z["horiz_sha"])
    assert out_sha(vert) == str(z["vert_sha"])


@pytest.mark.parametrize("path", small_golden_files(), ids=os.path.basename)
def test_stream_oracle_matches_golden_small(port, path):
    """The bounded-memory restatement (orc_compute_stream, which made the 4096x3000/512 fixture) reproduces the
    reference-made fixtures, every mode."""
    views, dc, gold, _ = load_small(path)
    for mode in range(3):
        got = port.compute_stream(views, dc, mode)
        assert np.array_equal(got, gold[mode]), "mode %d differs in %d px" % (mode, int((got != gold[mode]).sum()))


@pytest.mark.slow
def test_stream_oracle_matches_golden_c1(port):
    z = np.load(os.path.join(GOLDEN, "c1_640x480_dc192.npz"))
    (views, _), dc = synth.rig_c1(int(z["seed"]))
    for mode, key in enumerate(("multi_sha", "horiz_sha", "vert_sha")):
        assert out_sha(port.compute_stream(views, dc, mode)) == str(z[key])


@pytest.mark.parametrize("w,h,dc", [(40, 32, 264), (64, 48, 96)])
def test_stream_oracle_matches_full_oracle_wide(port, w, h, dc):
    """Above 256 disparities (where the reference's WTARight_SSE overflows) the two restatements agree."""
    rng = np.random.default_rng(w * h + dc)
    views = [rng.integers(0, 256, (h, w), dtype=np.uint8) for _ in range(5)]
    full = port.compute(views, dc)
    for mode in range(3):
        assert np.array_equal(port.compute_stream(views, dc, mode), full[mode])


def test_generator_reproduces_c5_inputs():
    z = np.load(os.path.join(GOLDEN, "c5_4096x3000_dc512.npz"))
    (views, _), dc = synth.rig_c5(int(z["seed"]))
    assert dc == int(z["dc"])
    assert views_sha(views) == str(z["views_sha"])


def test_synthetic_scene_is_recovered(port):
    """The generator warps in the direction the matcher searches: disparities come back."""
    views, gt = synth.make_rig(160, 120, 4, 40, seed=7, tiles=4)
    multi = port.compute(views, 48, modes=(True, False, False))[0]
    d = multi.astype(np.int64) // 255
    inner = (slice(8, -8), slice(8, -8))
    err = np.abs(d[inner] - gt[inner])
    assert np.median(err) <= 1
    assert (err <= 1).mean() > 0.85


def test_generator_is_deterministic():
    a, _ = synth.make_rig(64, 48, 2, 12, seed=11, tiles=3)
    b, _ = synth.make_rig(64, 48, 2, 12, seed=11, tiles=3)
    c, _ = synth.make_rig(64, 48, 2, 12, seed=12, tiles=3)
    assert views_sha(a) == views_sha(b) != views_sha(c)


@pytest.mark.parametrize("args", [(64, 48, 2, 12, 11, 3, False, 1.5), (96, 64, 2, 20, 9, 4, True, 0.8),
                                  (200, 148, 4, 64, 21, 10, True, 1.5), (320, 240, 8, 60, 5, 6, False, 0.8)])
def test_native_generator_is_byte_identical(args):
    """sister_synth_rig (the library's C port of make_rig) gives the same bytes as the numpy definition."""
    a_views, a_disp = synth._make_rig_native(*args)
    b_views, b_disp = synth.make_rig_numpy(*args)
    assert views_sha(a_views) == views_sha(b_views)
    assert np.array_equal(a_disp, b_disp)


def test_batch_shapes_follow_workload_rules():
    shapes = synth.batch_shapes(64, seed=3)
    assert len(shapes) == 64
    for w, h, dc in shapes:
        assert 320 <= w <= 2448 and 240 <= h <= 2048 and w % 16 == 0 and h % 16 == 0
        assert dc in (64, 128, 192, 256) and dc <= w // 4


def test_port_rejects_bad_geometry(port):
    views = [np.zeros((30, 40), np.uint8)] * 5  # h % 4 != 0
    with pytest.raises(RuntimeError):
        port.compute(views, 16)
    views = [np.zeros((32, 40), np.uint8)] * 5
    with pytest.raises(RuntimeError):
        port.compute(views, 12)  # dc % 8 != 0


# ---- stage-by-stage against the reference's own compiled code ---------------------------------

needs_ref = pytest.mark.skipif(not oracle.reference_available(), reason="reference tree / x86 host not available")


@pytest.fixture(scope="module")
def ref():
    return oracle.Ref()


@needs_ref
@pytest.mark.parametrize("shape", [(20, 24), (37, 40), (64, 48), (11, 13)])
def test_census_vs_ref(port, ref, shape):
    img = np.random.default_rng(shape[0]).integers(0, 256, shape, dtype=np.uint8)
    assert np.array_equal(port.census(img), ref.census(img))


@needs_ref
@pytest.mark.parametrize("H,W,D", [(20, 24, 8), (40, 64, 16), (64, 48, 32), (12, 40, 40)])
def test_cost_volume_and_wta_vs_ref(port, ref, H, W, D):
    rng = np.random.default_rng(H * W + D)
    x = rng.integers(0, 256, (H, W), dtype=np.uint8)
    y = rng.integers(0, 256, (H, W), dtype=np.uint8)
    vr = ref.ad_census(x, y, D)
    cx, cy = port.census(x), port.census(y)
    assert np.array_equal(port.cost_volume(cx, cy, D), vr)
    L, R = port.wta_lr(cx, cy, D)
    assert np.array_equal(L, ref.wta(vr, False))
    assert np.array_equal(R, ref.wta(vr, True))


@needs_ref
@pytest.mark.parametrize("H,W,D", [(20, 24, 8), (36, 20, 64), (48, 64, 16), (9, 8, 8), (64, 12, 32)])
def test_median_vs_ref(port, ref, H, W, D):
    a = np.random.default_rng(H + W).integers(0, D, (H, W)).astype(np.uint16)
    assert np.array_equal(port.median_inplace(a), ref.median_inplace(a.astype(np.float32)))


@needs_ref
@pytest.mark.parametrize("H,W,D", [(20, 24, 8), (40, 64, 16)])
def test_lrc_mask_vs_ref(port, ref, H, W, D):
    rng = np.random.default_rng(W)
    L = rng.integers(0, D, (H, W)).astype(np.uint16)
    R = rng.integers(0, D, (H, W)).astype(np.uint16)
    Lc = ref.lrcheck(L.astype(np.float32), R.astype(np.float32))
    expect = ((Lc > 0) & (np.arange(W)[None, :] >= D)).astype(np.uint8)
    assert np.array_equal(port.lrc_mask(L, R, D), expect)


@needs_ref
@pytest.mark.parametrize("H,W,D", [(12, 16, 8), (20, 24, 16), (33, 40, 32), (16, 48, 64)])
@pytest.mark.parametrize("kind", ["popcount", "special", "wide"])
def test_sgm_vs_ref(port, ref, H, W, D, kind):
    rng = np.random.default_rng(H * 7 + W + D)
    if kind == "popcount":
        C = rng.integers(0, 65, (H, W, D)).astype(np.uint16)
    elif kind == "special":  # 255 (substituted on first lines), sums above 255 (8-bit truncation)
        C = rng.choice(np.array([0, 5, 64, 255, 256, 300, 1020], np.uint16), (H, W, D))
    else:
        C = rng.integers(0, 1021, (H, W, D)).astype(np.uint16)
    assert np.array_equal(port.sgm(C), ref.sgm(C))


@needs_ref
@pytest.mark.parametrize("h,w,dc", [(16, 24, 8), (32, 40, 16), (40, 56, 24), (24, 96, 32)])
def test_compute_vs_ref_random(port, ref, h, w, dc):
    rng = np.random.default_rng(h * w * dc)
    views = [rng.integers(0, 256, (h, w), dtype=np.uint8) for _ in range(5)]
    got, want = port.compute(views, dc), ref.compute(views, dc)
    for k in range(3):
        assert np.array_equal(got[k], want[k])
