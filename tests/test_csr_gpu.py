"""CSR system matrix: built on the GPU from the forward projector's rule.

A must reproduce the on-the-fly projector and the oracle's system matrix, and
A^T must be exactly its transpose (same positions, bit-identical values)."""
import math

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import cpu_ref
from oracle import fut_ref as F
from synkrotomo_gb300 import phantom
from synkrotomo_gb300 import runtime as rt
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _scipy(m, transpose=False):
    p, i, v = (t.cpu().numpy() for t in m.arrays(transpose))
    shape = (m.cols, m.rows) if transpose else (m.rows, m.cols)
    return sp.csr_matrix((v, i, p), shape=shape)


@pytest.mark.parametrize("size,a,nr,dr", [(16, 12, None, 1.0), (32, 30, 46, 1.0), (40, 17, None, 0.5),
                                          (64, 64, None, 1.0), (24, 9, 40, 1.5)])
def test_csr_matches_oracle_and_transpose(gpu, size, a, nr, dr):
    g = phantom.geometry(size, a, numrhos=nr, deltarho=dr)
    m = rt.SystemMatrix(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, size)
    A = _scipy(m)
    AT = _scipy(m, transpose=True)
    assert A.shape == (a * g.numrhos, size * size) and m.nnz == A.nnz
    # exact transpose: same sparsity, bit-identical values, rows of A^T sorted by ray
    diff = (A.T.tocsr() - AT)
    assert diff.nnz == 0 or np.max(np.abs(diff.data)) == 0.0
    for r in range(0, AT.shape[0], max(1, AT.shape[0] // 50)):
        idx = AT.indices[AT.indptr[r]:AT.indptr[r + 1]]
        assert np.all(np.diff(idx) > 0)
    # the f32 reference's projection, and the FP64 oracle's matrix wherever the
    # oracle pair agrees (no ray along a pixel edge)
    x = phantom.ellipse_phantom(size, seed=size)
    ref32 = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, x)
    assert rel_l2(A @ x, ref32) < 1e-5
    O = F.fp_matrix(g.angles, g.rhozero, g.deltarho, g.numrhos, size)
    ref64 = O @ x.astype(np.float64)
    if rel_l2(ref32, ref64) < 1e-5:
        assert rel_l2(A @ x, ref64) < 1e-5
    # SpMV on the GPU = the on-the-fly projector
    xd = _dev(x)
    y = m.matvec(xd)
    fp = rt.forwardprojection(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, xd)
    assert rel_l2(y.cpu().numpy(), fp.cpu().numpy()) < 1e-5
    w = np.random.default_rng(1).random(m.rows).astype(np.float32)
    z = m.rmatvec(_dev(w)).cpu().numpy()
    assert rel_l2(z, AT @ w.astype(np.float64)) < 1e-6


def test_csr_config_sparse_scale(gpu):
    """N=512, 512 angles, 725 detectors: the sparse projector benchmark's matrix."""
    g = phantom.geometry(512, 512, numrhos=725)
    m = rt.SystemMatrix(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, 512)
    assert m.rows == 512 * 725 and m.cols == 512 * 512
    assert abs(m.nnz - 1.709e8) / 1.709e8 < 0.01
    rng = np.random.default_rng(2)
    x = _dev(rng.random(m.cols).astype(np.float32))
    y = _dev(rng.random(m.rows).astype(np.float32))
    ax = m.matvec(x)
    aty = m.rmatvec(y)
    lhs = float(torch.dot(ax.double(), y.double()))
    rhs = float(torch.dot(x.double(), aty.double()))
    assert abs(lhs - rhs) / abs(lhs) < 1e-6       # <Ax, y> = <x, A^T y>
    fp = rt.forwardprojection(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, x)
    assert rel_l2(ax.cpu().numpy(), fp.cpu().numpy()) < 1e-5


def test_spmv_csr32_caller_matrix(gpu):
    M = sp.random(300, 200, density=0.05, format="csr", random_state=0, dtype=np.float32)
    x = np.random.default_rng(0).random(200).astype(np.float32)
    ctx = rt.context()
    y = torch.empty(300, device="cuda")
    ptr = _dev(M.indptr.astype(np.int32))
    idx = _dev(M.indices.astype(np.int32))
    val = _dev(M.data.astype(np.float32))
    xd = _dev(x)
    rc = ctx.lib.synk_spmv_csr32(ctx.handle, 300, rt._ptr(ptr), rt._ptr(idx), rt._ptr(val), rt._ptr(xd), rt._ptr(y))
    ctx.check(rc, "spmv")
    assert rel_l2(y.cpu().numpy(), M @ x.astype(np.float64)) < 1e-6


def test_spmv_csr32_ragged_rows_and_nonfinite_x(gpu):
    """Rows of 0..300 entries (partial 128-entry chunks at every offset) and a
    non-finite x[0]: rows that do not hold column 0 stay finite and match the
    float64 product, rows that do are +inf, empty rows are 0."""
    rng = np.random.default_rng(1)
    cols = 400
    lens = [0, 1, 31, 32, 33, 96, 97, 127, 128, 129, 255, 256, 257, 300, 0, 5]
    indptr = np.concatenate([[0], np.cumsum(lens)]).astype(np.int32)
    idx = np.concatenate([np.sort(rng.choice(np.arange(1, cols), n, replace=False)) for n in lens]).astype(np.int32)
    idx[indptr[3]] = 0          # the row of 32 entries holds column 0
    val = rng.random(idx.size).astype(np.float32) + 0.5
    x = rng.random(cols).astype(np.float32)
    x[0] = np.inf
    rows = len(lens)
    y = torch.full((rows,), -1.0, device="cuda")
    ctx = rt.context()
    args = [_dev(indptr), _dev(idx), _dev(val), _dev(x)]
    rc = ctx.lib.synk_spmv_csr32(ctx.handle, rows, *[rt._ptr(t) for t in args], rt._ptr(y))
    ctx.check(rc, "spmv")
    got = y.cpu().numpy()
    for r in range(rows):
        sl = slice(indptr[r], indptr[r + 1])
        if r == 3:
            assert got[r] == np.inf
            continue
        ref = float(np.dot(val[sl].astype(np.float64), x[idx[sl]].astype(np.float64)))
        assert np.isfinite(got[r]), r
        assert abs(got[r] - ref) <= 1e-6 * max(abs(ref), 1.0), (r, got[r], ref)
