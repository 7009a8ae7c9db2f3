"""Serving loop (sister_server_*) with continuous admission: requests submitted from several host threads, and
requests submitted while others are on the GPU, must each equal the single-rig path bit for bit (the same
result alone and in the mix); several requests must actually be in flight at once; a full queue refuses
requests (backpressure) without disturbing the accepted ones; a wait that times out on the host reports the
request as pending and leaves its ticket valid; a request that alone exceeds the budget, or a malformed one, is
refused at submission while the others are served."""
import threading

import numpy as np
import pytest

import sister_gb300 as sg
from sister_gb300 import synth

pytestmark = pytest.mark.gpu

SHAPES = [(96, 64, 24), (128, 96, 40), (64, 48, 16), (160, 120, 64), (96, 64, 24), (200, 148, 72)]


def _rig(k, shapes=SHAPES, seed0=90):
    w, h, dc = shapes[k]
    views, _ = synth.make_rig(w, h, 2, dc - 6, seed=seed0 + k, tiles=4)
    return views, dc


def _single(views, dc, modes=(True, False, False)):
    ctx = sg.Context(0)
    ctx.load_views(views)
    ctx.set_max_disparity(dc)
    out = ctx.compute(*modes)
    ctx.close()
    return out


def test_server_concurrent_submitters_match_single_rig_path(gpu_lib, port):
    rigs = [_rig(k) for k in range(len(SHAPES))]
    want = [_single(v, dc)[0] for v, dc in rigs]
    for k, (v, dc) in enumerate(rigs):  # the single-rig path itself against the oracle for these shapes
        assert np.array_equal(want[k], port.compute(v, dc, modes=(True, False, False))[0]), "rig %d" % k
    srv = sg.Server(0, 1 << 30)
    tickets = [None] * len(rigs)

    def submitter(ks):
        for k in ks:
            tickets[k] = srv.submit(rigs[k][0], rigs[k][1])

    th = [threading.Thread(target=submitter, args=(list(range(i, len(rigs), 3)),)) for i in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k, t in enumerate(tickets):
        out, lat = srv.wait(t)
        assert lat > 0
        assert np.array_equal(out[0], want[k]), "request %d: %d px differ" % (k, int((out[0] != want[k]).sum()))
    st = srv.stats()
    assert st["completed"] == len(rigs) and st["admitted"] == len(rigs) and st["rejected"] == 0
    srv.close()


def test_requests_overlap_and_match_alone(gpu_lib):
    """Larger rigs keep the GPU busy for milliseconds each; the ones submitted meanwhile are admitted and run
    beside them (peak in flight > 1), and every result equals the same rig computed alone, in all modes asked."""
    shapes = [(640, 480, 128), (320, 240, 64), (480, 320, 96), (640, 480, 128), (256, 192, 64), (320, 240, 64),
              (480, 320, 96), (256, 192, 64)]
    rigs = [_rig(k, shapes, seed0=500) for k in range(len(shapes))]
    modes = [(True, False, False), (True, True, True), (False, False, True), (True, False, False),
             (True, True, False), (True, False, False), (False, True, False), (True, False, True)]
    want = [_single(v, dc, m) for (v, dc), m in zip(rigs, modes)]
    srv = sg.Server(0, 8 << 30, max_inflight=4)
    tickets = [srv.submit(v, dc, m) for (v, dc), m in zip(rigs, modes)]
    for k, t in enumerate(tickets):
        out, _ = srv.wait(t)
        for m in range(3):
            if want[k][m] is None:
                assert out[m] is None
            else:
                assert np.array_equal(out[m], want[k][m]), "request %d mode %d: %d px differ" % (
                    k, m, int((out[m] != want[k][m]).sum()))
    assert srv.stats()["peak_inflight"] >= 2
    srv.close()


def test_wide_stride_requests_match_oracle(gpu_lib, port):
    """Requests with d-strides above 256 (wider records and cost batches in the aggregation) beside a narrow one in
    one server, against the oracle."""
    shapes = [(200, 120, 264), (160, 96, 64), (128, 96, 312)]
    rigs = [_rig(k, shapes, seed0=700) for k in range(len(shapes))]
    srv = sg.Server(0, 4 << 30)
    tickets = [srv.submit(v, dc) for v, dc in rigs]
    for k, t in enumerate(tickets):
        out, _ = srv.wait(t)
        want = port.compute(rigs[k][0], rigs[k][1], modes=(True, False, False))[0]
        assert np.array_equal(out[0], want), "request %d: %d px differ" % (k, int((out[0] != want).sum()))
    srv.close()


def test_full_queue_refuses_and_pending_wait(gpu_lib):
    views, dc = _rig(0, [(640, 480, 128)], seed0=77)
    want = _single(views, dc)[0]
    srv = sg.Server(0, 4 << 30, max_inflight=1, max_queue=1)
    accepted, busy = [], 0
    for _ in range(6):
        try:
            accepted.append(srv.submit(views, dc))
        except sg.SisterError as e:
            assert e.code == sg.SISTER_EBUSY, str(e)
            busy += 1
    assert busy >= 1 and accepted
    with pytest.raises(TimeoutError):
        srv.wait(accepted[-1], 0)  # still queued or running: pending, the ticket stays valid
    for t in accepted:
        out, _ = srv.wait(t)
        assert np.array_equal(out[0], want)
    assert srv.stats()["rejected"] == busy
    srv.close()


def test_server_refuses_request_beyond_budget_and_malformed(gpu_lib):
    views, _ = synth.make_rig(160, 120, 4, 40, seed=3, tiles=4)
    srv = sg.Server(0, 16 << 20)
    with pytest.raises(sg.SisterError) as ei:
        srv.submit(views, 64)  # ~30 MB (the cost volume of 288 x 248 padded pixels alone is 9 MB)
    assert ei.value.code == sg.SISTER_EBUDGET
    with pytest.raises(sg.SisterError) as ei:
        srv.submit(views, 60)  # max disparity not a multiple of 8
    assert ei.value.code == sg.SISTER_EINVAL
    small, _ = synth.make_rig(64, 48, 2, 12, seed=4, tiles=3)
    out, _ = srv.wait(srv.submit(small, 16))
    assert np.array_equal(out[0], _single(small, 16)[0])
    srv.close()
