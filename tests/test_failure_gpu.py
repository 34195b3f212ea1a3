"""Failure detection on the GPU without a GPU fault.

The persistent SIRT kernel's grid barrier waits with a time limit.  Here the
barrier is made to wait for one block more than the cooperative launch has
(a count that can never be reached), with a 20 ms limit: every block gives
up after 20 ms, records SYNK_ETIMEOUT and returns.  The test checks that the
next synk_context_sync() reports it, that the sync clears it, and that the
same context then solves the N=128 configuration exactly as before.  Nothing
traps, faults or waits without a bound.
"""
import numpy as np
import pytest
import torch

from synkrotomo_gb300 import _lib, phantom
from synkrotomo_gb300 import runtime as rt

pytestmark = pytest.mark.gpu


def _cfg0(seed=0):
    g = phantom.geometry(128, 128)
    img = torch.from_numpy(phantom.ellipse_phantom(128, seed)).cuda()
    ang = torch.from_numpy(g.angles).cuda()
    b = rt.forwardprojection(ang, g.rhozero, g.deltarho, g.numrhos, img)
    return g, ang, b


def test_barrier_timeout_is_reported_and_the_context_recovers(gpu):
    ctx = rt.context()
    g, ang, b = _cfg0()
    full = rt.resident_blocks()
    assert full > 0
    want, _, _ = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 128, 1, None, b, 30, grid_blocks=full)
    ctx.sync()
    want = want.clone()

    ctx.set_barrier_limit(20_000_000, missing_blocks=1)
    try:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 128, 1, None, b, 30, grid_blocks=full)
        t1.record()
        with pytest.raises(rt.SynkError) as e:
            ctx.sync()
        assert e.value.code == _lib.SYNK_ETIMEOUT
        assert "timed out" in str(e.value)
        # every block gave up at the first barrier, after about the 20 ms limit
        assert 15.0 < t0.elapsed_time(t1) < 2000.0
    finally:
        ctx.set_barrier_limit(2_000_000_000, 0)

    ctx.sync()          # the status was cleared by the failing sync
    got, _, done = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 128, 1, None, b, 30, grid_blocks=full)
    ctx.sync()
    assert torch.equal(got, want)
    assert int(done.item()) == 30


def test_barrier_limit_rejects_out_of_range_values(gpu):
    ctx = rt.context()
    with pytest.raises(ValueError):
        ctx.set_barrier_limit(10, 0)                 # below 1 us
    with pytest.raises(ValueError):
        ctx.set_barrier_limit(2_000_000_000, -1)
    ctx.set_barrier_limit()                          # the default stands
    g, ang, b = _cfg0(1)
    x, _, _ = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 128, 1, None, b, 5,
                             grid_blocks=rt.resident_blocks())
    ctx.sync()
    assert np.isfinite(x.cpu().numpy()).all()
