"""Batched rigs (sister_batch_run): every rig of a batch must equal the single-rig path (itself checked
against the oracle and the compiled reference) bit for bit, whatever the mix of sizes, disparity ranges,
modes and channel counts, and however the budget splits the batch into waves."""
import numpy as np
import pytest

import sister_gb300 as sg
from sister_gb300 import synth

pytestmark = pytest.mark.gpu

# (w, h, dmin, dmax, dc, modes, bgr): mixed sizes and all three d-stride classes below 256
MIX = [
    (96, 64, 2, 20, 24, (True, False, False), False),
    (160, 120, 4, 56, 64, (True, True, True), False),
    (128, 96, 2, 30, 40, (False, True, False), True),
    (200, 148, 4, 64, 72, (True, False, True), False),
    (64, 48, 1, 12, 16, (True, True, False), False),
    (240, 160, 6, 110, 128, (True, False, False), False),
]


def _rigs(seed0=40):
    rigs = []
    for k, (w, h, lo, hi, dc, modes, bgr) in enumerate(MIX):
        views, _ = synth.make_rig(w, h, lo, hi, seed=seed0 + k, tiles=4)
        if bgr:
            views = [np.stack([v, np.roll(v, 1, axis=1), v[::-1, :]], axis=2) for v in views]
        rigs.append((views, dc, modes))
    return rigs


def _single(rig):
    views, dc, modes = rig
    ctx = sg.Context(0)
    ctx.load_views(views)
    ctx.set_max_disparity(dc)
    out = ctx.compute(*modes)
    ctx.close()
    return out


def _check(got, want):
    for k, (g, w) in enumerate(zip(got, want)):
        for m in range(3):
            if w[m] is None:
                assert g[m] is None
            else:
                assert np.array_equal(g[m], w[m]), "rig %d mode %d: %d px differ" % (k, m, int((g[m] != w[m]).sum()))


def test_batch_matches_single_rig_path(gpu_lib):
    rigs = _rigs()
    want = [_single(r) for r in rigs]
    b = sg.Batch(0, 0)
    _check(b.run(rigs), want)
    _check(b.run(rigs), want)  # the arena is reused; nothing of the previous call may leak into the next
    b.close()


def test_batch_matches_oracle(gpu_lib, port):
    """The batched outputs against the oracle directly (not only through the single-rig path): every gray rig of
    the mix, in every mode it asks for, in one batch."""
    rigs = [r for r, spec in zip(_rigs(seed0=90), MIX) if not spec[6]]
    b = sg.Batch(0, 0)
    got = b.run(rigs)
    b.close()
    for k, ((views, dc, modes), g) in enumerate(zip(rigs, got)):
        want = port.compute(views, dc, modes=modes)
        for m in range(3):
            if modes[m]:
                assert np.array_equal(g[m], want[m]), "rig %d mode %d: %d px differ" % (
                    k, m, int((g[m] != want[m]).sum()))


def test_batch_benchmark_shapes_match_oracle(gpu_lib, port):
    """The four smallest rigs of the benchmarked 64-rig uneven batch (same shapes and seeds as its batched leg),
    batched together with two of its larger rigs, against the oracle: the benchmark's own shapes meet the oracle,
    not only the single-rig path."""
    shapes = synth.batch_shapes(64, seed=3)
    cells = [((w + 2 * dc) * (h + 2 * dc) * dc, k) for k, (w, h, dc) in enumerate(shapes)]
    pick = [k for _, k in sorted(cells)[:4]] + [k for _, k in sorted(cells)[30:32]]
    rigs = [synth.rig_for_shape(*shapes[k], seed=1000 + k) for k in pick]
    b = sg.Batch(0, 0)
    got = b.run([(views, dc) for (views, _), dc in rigs])
    b.close()
    for k, (((views, _), dc), g) in enumerate(zip(rigs, got)):
        if k >= 4:
            continue  # the larger rigs only share the batch; the oracle checks the four small ones
        want = port.compute(views, dc, modes=(True, False, False))[0]
        assert np.array_equal(g[0], want), "shape %s: %d px differ" % (shapes[pick[k]], int((g[0] != want).sum()))


def test_batch_wide_strides_match_oracle(gpu_lib, port):
    """d-strides above 256 (their own aggregation launches, with 12-row bands and 2-pixel cost copies at 512)
    batched with narrower ones, against the oracle."""
    specs = [(200, 120, 4, 240, 264), (160, 96, 2, 56, 64), (128, 96, 4, 290, 312), (96, 64, 2, 20, 24)]
    rigs = []
    for k, (w, h, lo, hi, dc) in enumerate(specs):
        views, _ = synth.make_rig(w, h, lo, hi, seed=800 + k, tiles=4)
        rigs.append((views, dc))
    b = sg.Batch(0, 0)
    got = b.run(rigs)
    b.close()
    for k, ((views, dc), g) in enumerate(zip(rigs, got)):
        want = port.compute(views, dc, modes=(True, False, False))[0]
        assert np.array_equal(g[0], want), "rig %d (dc %d): %d px differ" % (k, dc, int((g[0] != want).sum()))


def test_batch_waves_under_a_small_budget(gpu_lib):
    rigs = _rigs(seed0=70)
    want = [_single(r) for r in rigs]
    need = max(sg.Batch.rig_bytes(r[0][0].shape[1], r[0][0].shape[0], r[1], sum(r[2])) for r in rigs)
    b = sg.Batch(0, need + (24 << 20))  # room for about one rig per wave
    _check(b.run(rigs), want)
    b.close()


def test_batch_rejects_oversized_rig_and_bad_geometry(gpu_lib):
    views, _ = synth.make_rig(160, 120, 4, 40, seed=5, tiles=4)
    need = sg.Batch.rig_bytes(160, 120, 64, 1)
    b = sg.Batch(0, need // 2)
    with pytest.raises(sg.SisterError) as ei:
        b.run([(views, 64)])  # twice the budget for one mode
    assert ei.value.code == sg.SISTER_EBUDGET
    with pytest.raises(sg.SisterError) as ei:
        b.run([(views, 60)])  # not a multiple of 8
    assert ei.value.code == sg.SISTER_EINVAL
    b.close()
