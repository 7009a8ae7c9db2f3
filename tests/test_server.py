"""Serving loop (sister_server_*): requests submitted from several host threads are computed in dynamic
batches; every output must equal the single-rig path bit for bit, latencies are reported, and a request that
alone exceeds the budget is refused at submission."""
import threading

import numpy as np
import pytest

import sister_gb300 as sg
from sister_gb300 import synth

pytestmark = pytest.mark.gpu

SHAPES = [(96, 64, 24), (128, 96, 40), (64, 48, 16), (160, 120, 64), (96, 64, 24), (200, 148, 72)]


def _rig(k):
    w, h, dc = SHAPES[k]
    views, _ = synth.make_rig(w, h, 2, dc - 6, seed=90 + k, tiles=4)
    return views, dc


def _single(views, dc):
    ctx = sg.Context(0)
    ctx.load_views(views)
    ctx.set_max_disparity(dc)
    out = ctx.compute(True, False, False)[0]
    ctx.close()
    return out


def test_server_concurrent_submitters_match_single_rig_path(gpu_lib):
    rigs = [_rig(k) for k in range(len(SHAPES))]
    want = [_single(v, dc) for v, dc in rigs]
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
    assert st["rigs"] == len(rigs) and 1 <= st["batches"] <= len(rigs)
    srv.close()


def test_server_refuses_request_beyond_budget(gpu_lib):
    views, _ = synth.make_rig(160, 120, 4, 40, seed=3, tiles=4)
    srv = sg.Server(0, 40 << 20)
    with pytest.raises(sg.SisterError) as ei:
        srv.submit(views, 64)  # ~44 MB
    assert ei.value.code == sg.SISTER_EBUDGET
    small, _ = synth.make_rig(64, 48, 2, 12, seed=4, tiles=3)
    out, _ = srv.wait(srv.submit(small, 16))
    assert np.array_equal(out[0], _single(small, 16))
    srv.close()
