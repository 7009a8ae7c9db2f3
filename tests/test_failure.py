"""Failure paths on the GPU, made to happen without faulting anything: every device-side wait of the library is
bounded, so a wait that runs out raises the device error flag, the kernel finishes, and the call returns
SISTER_ETIMEOUT. Here the wait limit is lowered to 1 microsecond (SISTER_TUNE_WAIT_LIMIT_US) so that the band
hand-off waits of the aggregation (a later band waits hundreds of microseconds for the band above) run out on a
rig of many bands; the same context must then compute bit-exactly again with the default limit."""
import numpy as np
import pytest

import sister_gb300 as sg
from sister_gb300 import synth

pytestmark = pytest.mark.gpu


def test_expired_wait_reports_timeout_and_context_recovers(gpu_lib, port):
    w, h, dc = 96, 320, 32  # padded 160 x 384: with 4-row bands, 96 bands per pass
    views, _ = synth.make_rig(w, h, 2, 24, seed=41, tiles=4)
    want = port.compute(views, dc, modes=(True, False, False))[0]
    ctx = sg.Context(0)
    try:
        ctx.load_views(views)
        ctx.set_max_disparity(dc)
        ctx.tune_set(sg.TUNE_SGM_ROWS, 4)
        ctx.tune_set(sg.TUNE_WAIT_LIMIT_US, 1)
        assert ctx.tune_get(sg.TUNE_WAIT_LIMIT_US) == 1
        with pytest.raises(sg.SisterError) as e:
            ctx.compute(True, False, False)
        assert e.value.code == sg.SISTER_ETIMEOUT, str(e.value)
        ctx.tune_set(sg.TUNE_WAIT_LIMIT_US, 0)  # back to the default limit
        assert ctx.tune_get(sg.TUNE_WAIT_LIMIT_US) == 2000000
        for _ in range(2):
            got = ctx.compute(True, False, False)[0]
            assert np.array_equal(got, want), "%d px differ after the timeout" % int((got != want).sum())
    finally:
        ctx.close()


def test_wait_limit_rejects_negative(gpu_lib):
    ctx = sg.Context(0)
    try:
        with pytest.raises(sg.SisterError) as e:
            ctx.tune_set(sg.TUNE_WAIT_LIMIT_US, -1)
        assert e.value.code == sg.SISTER_EINVAL
    finally:
        ctx.close()
