"""The backprojection entry point that allocates nothing.

Some callers cannot let the library allocate device memory: programs that
reserve all free device memory for their own allocator at start-up, and
acquisition loops that must not enter the CUDA allocator while frames stream.
synk_backprojection_noalloc serves them with its scratch in a fixed device
array.  This file is collected last on purpose (pytest orders files by name),
so a failure here does not stop the other tests from running first.
"""
import numpy as np
import pytest
import torch

from oracle import cpu_ref
from synkrotomo_gb300 import _lib, phantom
from synkrotomo_gb300 import runtime as rt
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu

MAX_ANGLES = 8192   # SYNK_NOALLOC_MAX_ANGLES in include/synk.h


def _noalloc(ctx, out, ang, g, size, sino):
    return ctx.lib.synk_backprojection_noalloc(ctx.handle, rt._ptr(out), rt._ptr(ang), ang.numel(),
                                               g.rhozero, g.deltarho, int(size), rt._ptr(sino), sino.numel())


def _regular(ctx, out, ang, g, size, sino):
    return ctx.lib.synk_backprojection(ctx.handle, rt._ptr(out), rt._ptr(ang), ang.numel(),
                                       g.rhozero, g.deltarho, int(size), rt._ptr(sino), sino.numel())


def _pair(ctx, size, n_angles, nr, seed):
    g = phantom.geometry(size, n_angles, numrhos=nr)
    ang = torch.from_numpy(g.angles).cuda()
    sino_h = np.random.default_rng(seed).random(g.n_rays).astype(np.float32)
    sino = torch.from_numpy(sino_h).cuda()
    want = torch.empty(size * size, device="cuda")
    got = torch.full((size * size,), float("nan"), device="cuda")
    ctx.check(_regular(ctx, want, ang, g, size, sino), "synk_backprojection")
    ctx.check(_noalloc(ctx, got, ang, g, size, sino), "synk_backprojection_noalloc")
    ctx.sync()
    return g, sino_h, got.cpu().numpy(), want.cpu().numpy()


def test_noalloc_backprojection_matches_regular_entry_twice(gpu):
    ctx = rt.context()
    # two calls in a row with different geometries, so the second call must
    # overwrite everything the first one left in the shared scratch array
    for size, n_angles, nr, seed in ((64, 90, None, 0), (96, 37, 150, 1)):
        _, _, got, want = _pair(ctx, size, n_angles, nr, seed)
        assert rel_l2(got, want) < 1e-5


@pytest.mark.parametrize("size,n_angles", [(48, 300), (32, 1500), (16, MAX_ANGLES)])
def test_noalloc_backprojection_many_angles(gpu, size, n_angles):
    """300 angles run the 8-pixel kernel, 1500 the separate geometry launch, and
    8192 fills the scratch array to its limit; each matches the regular entry
    point and the FP32 oracle."""
    ctx = rt.context()
    g, sino, got, want = _pair(ctx, size, n_angles, None, n_angles)
    assert rel_l2(got, want) < 1e-5
    ref = cpu_ref.backprojection(g.angles, g.rhozero, g.deltarho, size, sino)
    assert rel_l2(got, ref) < 1e-5
    # and once more, after a call with fewer angles has overwritten the start of the array
    _pair(ctx, 64, 90, None, 5)
    _, _, again, _ = _pair(ctx, size, n_angles, None, n_angles)
    np.testing.assert_array_equal(again, got)


def test_noalloc_rejects_too_many_angles(gpu):
    ctx = rt.context()
    g = phantom.geometry(16, 4)
    ang = torch.zeros(MAX_ANGLES + 1, device="cuda")
    sino = torch.zeros((MAX_ANGLES + 1) * g.numrhos, device="cuda")
    out = torch.empty(16 * 16, device="cuda")
    rc = _noalloc(ctx, out, ang, g, 16, sino)
    assert rc == _lib.SYNK_EINVAL
    assert b"at most 8192 angles" in ctx.lib.synk_context_get_error(ctx.handle)
