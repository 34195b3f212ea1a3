"""Parity of the persistent CUDA SIRT with the oracle.

Bar (from the project's accuracy targets): plain SIRT within 1e-5 relative L2
of the FP32 reference and within 1e-4 of the FP64 oracle.
"""
import math

import numpy as np
import pytest
import torch

from oracle import cpu_ref
from oracle import fut_ref as F
from synkrotomo_gb300 import phantom
from synkrotomo_gb300 import runtime as rt
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _problem(size, a, seed, nr=None, noise=0.01, arc=math.pi):
    g = phantom.geometry(size, a, numrhos=nr, arc=arc)
    img = phantom.ellipse_phantom(size, seed)
    b = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
    if noise:
        b = phantom.add_noise(b, seed, noise)
    return g, img, b


def test_sirt_config0_parity(gpu):
    """N=128, 128 angles, 182 detectors, 1 % noise, 200 iterations."""
    g, _, b = _problem(128, 128, seed=0)
    x0 = np.zeros(128 * 128, np.float32)
    x = rt.sirt(_dev(g.angles), g.rhozero, g.deltarho, _dev(x0), _dev(b), 200).cpu().numpy()
    ref32 = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, x0, b, 200)
    ops = F.SirtOperators(g.angles, g.rhozero, g.deltarho, g.numrhos, 128)
    ref64 = ops.iterate(x0, b, 200)
    assert rel_l2(x, ref32) < 1e-5
    assert rel_l2(x, ref64) < 1e-4


@pytest.mark.parametrize("size,a,nr,its", [(16, 12, None, 20), (32, 30, None, 50), (64, 17, 91, 30), (24, 40, 60, 25)])
def test_sirt_small_geometries(gpu, size, a, nr, its):
    g, img, b = _problem(size, a, seed=size, nr=nr)
    x0 = (0.1 * img).astype(np.float32)       # a non-zero start
    x = rt.sirt(_dev(g.angles), g.rhozero, g.deltarho, _dev(x0), _dev(b), its).cpu().numpy()
    ref32 = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, x0, b, its)
    assert rel_l2(x, ref32) < 1e-5


def test_sirt_zero_iterations_returns_start(gpu):
    g, img, b = _problem(32, 10, seed=2)
    x = rt.sirt(_dev(g.angles), g.rhozero, g.deltarho, _dev(img), _dev(b), 0).cpu().numpy()
    np.testing.assert_array_equal(x, img)


@pytest.mark.parametrize("fs,bs", [(1, 1), (2, 4), (8, 8), (4, 2)])
def test_work_splits_agree(gpu, fs, bs):
    g, _, b = _problem(64, 48, seed=4)
    ang, bd = _dev(g.angles), _dev(b)
    x, res, done = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 64, 1, None, bd, 40,
                                  fp_split=fs, bp_split=bs, residuals=True)
    ref32 = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(64 * 64, np.float32), b, 40)
    assert rel_l2(x.cpu().numpy(), ref32) < 1e-5
    assert int(done.item()) == 40


def test_residual_history_and_stopping_rule(gpu):
    # even detector count: half-integer rhozero, no ray on a pixel edge, so the
    # FP64 oracle and the f32 reference describe the same system
    g, _, b = _problem(64, 60, seed=7, nr=92, noise=0.0)
    ang, bd = _dev(g.angles), _dev(b)
    x, res, done = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 64, 1, None, bd, 60, residuals=True)
    ops = F.SirtOperators(g.angles, g.rhozero, g.deltarho, g.numrhos, 64)
    hist = []
    ops.iterate(np.zeros(64 * 64, np.float32), b, 60, hist)
    r = res.cpu().numpy()[0]
    np.testing.assert_allclose(r, hist, rtol=1e-4)
    # stop at the first iterate whose residual is below the 20th iterate's
    tol = float(hist[20]) * 1.0001
    x2, res2, done2 = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 64, 1, None, bd, 60, tol=tol,
                                     residuals=True)
    k = int(done2.item())
    assert k == next(i for i, v in enumerate(hist) if v <= tol)
    xk = ops.iterate(np.zeros(64 * 64, np.float32), b, k)
    assert rel_l2(x2.cpu().numpy(), xk) < 1e-4


def test_sirt_slices_match_single_slice_runs(gpu):
    size, a, ns = 32, 24, 5
    g = phantom.geometry(size, a)
    vol = phantom.ellipsoid_volume(size, ns, seed=1)
    sinos = np.stack([cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, vol[i])
                      for i in range(ns)])
    x, _, _ = rt.sirt_slices(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, size, ns, None,
                             _dev(sinos.ravel()), 15)
    x = x.cpu().numpy().reshape(ns, -1)
    for i in range(ns):
        ref = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(size * size, np.float32), sinos[i], 15)
        assert rel_l2(x[i], ref) < 1e-5


def test_sirt3d_matches_reference_semantics(gpu):
    size, a = 16, 10
    g = phantom.geometry(size, a, numrhos=24)
    rhos = (g.rhozero + np.arange(24) * g.deltarho).astype(np.float32)
    proj = np.random.default_rng(3).random(size * a * 24).astype(np.float32)
    x = rt.sirt3d(_dev(g.angles), _dev(rhos), _dev(proj), 8, size).cpu().numpy()
    ref = cpu_ref.sirt3d(g.angles, rhos, proj, 8, size)
    assert x.shape == (size ** 3,)
    assert rel_l2(x, ref) < 1e-5


def test_phase_split_engine_matches_persistent(gpu):
    """grid_blocks=-1 runs one launch per phase and iteration.  With the same
    work splits the same items compute the same values, so without a stopping
    rule the iterates are bit-identical to the persistent kernel's; with one,
    every slice stops at the same iteration (the loop then ends on the host's
    check of the active count after iteration 16, 32, ...)."""
    size, a, ns, its = 48, 40, 6, 45
    g = phantom.geometry(size, a)
    vol = phantom.ellipsoid_volume(size, ns, seed=3)
    sinos = np.stack([cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, vol[i])
                      for i in range(ns)])
    ang, bd = _dev(g.angles), _dev(sinos.ravel())
    full = rt.resident_blocks()
    kw = dict(fp_split=2, bp_split=4)
    xp, rp, dp = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, residuals=True,
                                grid_blocks=full, **kw)
    xs, rs, ds = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, residuals=True,
                                grid_blocks=-1, **kw)
    assert torch.equal(xp, xs)
    assert torch.equal(dp, ds)
    np.testing.assert_allclose(rs.cpu().numpy(), rp.cpu().numpy(), rtol=1e-12)
    ref = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(size * size, np.float32), sinos[2], its)
    assert rel_l2(xs.cpu().numpy().reshape(ns, -1)[2], ref) < 1e-5
    # stopping rule: per-slice stops between iteration 8 and 30
    hist = rp.cpu().numpy()
    tol = float(np.median(hist[:, 20]))
    xp2, _, dp2 = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, tol=tol,
                                 grid_blocks=full, **kw)
    xs2, _, ds2 = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, tol=tol,
                                 grid_blocks=-1, **kw)
    assert torch.equal(dp2, ds2)
    assert torch.equal(xp2, xs2)
    assert int(ds2.min()) < its and int(ds2.max()) > 16


def test_phase_split_engine_uneven_batch(gpu):
    specs = [(64, 60, 20), (32, 90, 35), (48, 17, 10)]
    probs, refs = [], []
    for i, (size, a, its) in enumerate(specs):
        g, _, b = _problem(size, a, seed=30 + i)
        probs.append(rt.Problem(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, size, _dev(b), its))
        refs.append(cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(size * size, np.float32), b, its))
    rt.sirt_batch(probs, grid_blocks=-1)
    for p, ref, spec in zip(probs, refs, specs):
        assert rel_l2(p.out.cpu().numpy(), ref) < 1e-5, spec
        assert int(p.done.item()) == spec[2]
    with pytest.raises(ValueError):
        rt.sirt_batch(probs, grid_blocks=-2)


def test_phase_split_engine_large_stack_matches_persistent(gpu):
    """Above 6e7 work per iteration a single problem runs on the projectors'
    grids: the forward phase in sirt_fp_stack_kernel (the per-ray values of
    the generic phase) and the backward phase in sirt_bp_stack_kernel (32 x 64
    pixel tiles, the residual as detector pairs, the same angle order).  A
    pixel's detector coordinate comes from its thread's first row, so the
    iterates agree with the persistent kernel's to rounding, slice by slice,
    and with the oracle; with a stopping rule every slice stops at the same
    iteration."""
    size, a, ns, its = 256, 180, 4, 12
    g = phantom.geometry(size, a)
    vol = phantom.ellipsoid_volume(size, ns, seed=5)
    sinos = np.stack([cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, vol[i])
                      for i in range(ns)])
    ang, bd = _dev(g.angles), _dev(sinos.ravel())
    assert ns * a * size * (size + g.numrhos) > 6e7
    for fs, bs in ((2, 4), (8, 1), (0, 0)):
        xp, rp, _ = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, residuals=True,
                                   fp_split=fs, bp_split=bs, grid_blocks=rt.resident_blocks())
        xs, rs, _ = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, residuals=True,
                                   fp_split=fs, bp_split=bs, grid_blocks=-1)
        xp_, xs_ = xp.cpu().numpy().reshape(ns, -1), xs.cpu().numpy().reshape(ns, -1)
        for z in range(ns):
            assert rel_l2(xs_[z], xp_[z]) < 1e-6, (fs, bs, z)
        np.testing.assert_allclose(rs.cpu().numpy(), rp.cpu().numpy(), rtol=1e-5)
    ref = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(size * size, np.float32), sinos[1], its)
    assert rel_l2(xs.cpu().numpy().reshape(ns, -1)[1], ref) < 1e-5
    hist = rp.cpu().numpy()
    tol = float(np.median(hist[:, 6])) * 1.003
    _, _, dp = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, tol=tol,
                              grid_blocks=rt.resident_blocks())
    xs2, _, ds = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, size, ns, None, bd, its, tol=tol,
                                grid_blocks=-1)
    assert torch.equal(dp, ds)
    assert int(ds.min()) < its
    for z in range(ns):
        k = int(ds[z].item())
        refk = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(size * size, np.float32), sinos[z], k)
        assert rel_l2(xs2.cpu().numpy().reshape(ns, -1)[z], refk) < 1e-5, z