"""Pins of the oracle (CPU only).

The reference ships no expected FP/BP/SIRT outputs; what it does ship are the
known-answer tests of archive/line_lib.fut:1-57 (chord length of a ray with a
pixel on an 8x8 grid, rhozero -5.5, deltarho 1) and
archive/projection_lib.fut:1-41 (index of a pixel's first detector).  The
archive writes rays as rho = x*cos + y*sin; the current code
(forwardprojection.fut:26-29) as rho = x*cos - y*sin, so a KAT ray (theta,
rho) is the current ray (pi - theta, -rho).
"""
import math

import numpy as np
import pytest

from oracle import cpu_ref
from oracle import fut_ref as F
from synkrotomo_gb300 import phantom
from tests.conftest import rel_l2

# archive/line_lib.fut:1-57: (pixel, angle) -> [chord with rhomin, chord with rhomin+1]
LINE_LIB_KATS = [
    (19, 0.0, [1.0, 0.0]),
    (27, 1.57079632679, [1.0, 0.0]),
    (45, 0.78539816339, [0.17157287525, 0.65685424949]),
    (36, 0.78539816339, [1.0, 0.0]),
    (27, 0.78539816339, [1.0, 0.0]),
    (42, 2.35619449019, [0.17157287525, 0.65685424949]),
    (21, 2.35619449019, [0.65685424949, 0.17157287525]),
    (18, 0.78539816339, [0.65685424949, 0.17157287525]),
]

# archive/projection_lib.fut:1-41: (rhos, angles, angleindex, size, pixel) -> index
PROJ_RHOS = [-1.5, -0.5, 0.5, 1.5]
PROJ_ANGLES = [0.0, 0.785398, 1.5708, 2.35619]
PROJECTION_LIB_KATS = [(1, 4, 10, 6), (3, 4, 9, 14), (3, 4, 6, 13), (1, 4, 5, 5)]


def _kat_pixel(pix, size):
    # archive/line_lib.fut:135-140 lowerleftpixelpoint
    y = pix // size
    x = pix - size * y
    return x - size // 2, y - size // 2


@pytest.mark.parametrize("pix,angle,expected", LINE_LIB_KATS)
def test_line_lib_kat(pix, angle, expected):
    th = float(np.float32(angle))
    xmin, ymin = _kat_pixel(pix, 8)
    # archive convention: normal (cos, sin); first detector per backprojection.fut:50-53
    s = F.first_detector(math.cos(th), math.sin(th), xmin, ymin, -5.5, 1.0)
    rhos = [-5.5 + s, -5.5 + s + 1.0]
    theta_cur = np.array([np.float32(math.pi - th)], np.float32)
    A = F.fp_matrix(theta_cur, -5.5, 1.0, 12, 8).toarray()
    B = F.bp_matrix(theta_cur, -5.5, 1.0, 12, 8).toarray()
    pixel = (ymin + 4) * 8 + (xmin + 4)
    for rho, want in zip(rhos, expected):
        det = int(round(-rho + 5.5))
        assert A[det, pixel] == pytest.approx(want, abs=2e-7), ("fp rule", rho)
        assert B[pixel, det] == pytest.approx(want, abs=2e-7), ("bp rule", rho)


@pytest.mark.parametrize("angleindex,size,pixel,expected", PROJECTION_LIB_KATS)
def test_projection_lib_kat(angleindex, size, pixel, expected):
    rhozero = PROJ_RHOS[0]
    deltarho = PROJ_RHOS[1] - PROJ_RHOS[0]
    th = float(np.float32(PROJ_ANGLES[angleindex]))
    xmin, ymin = _kat_pixel(pixel, size)
    s = F.first_detector(math.cos(th), math.sin(th), xmin, ymin, rhozero, deltarho)
    assert angleindex * len(PROJ_RHOS) + int(s) == expected


@pytest.mark.parametrize("size,n_angles", [(32, 30), (128, 128), (24, 7)])
def test_fp32_restatement_matches_fp64_oracle(size, n_angles):
    g = phantom.geometry(size, n_angles)
    img = phantom.ellipse_phantom(size, seed=size)
    s64 = F.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
    s32 = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
    assert rel_l2(s32, s64) < 2e-6
    y = np.random.default_rng(size).random(g.n_rays).astype(np.float32)
    b64 = F.backprojection(g.angles, g.rhozero, g.deltarho, size, y)
    b32 = cpu_ref.backprojection(g.angles, g.rhozero, g.deltarho, size, y)
    assert rel_l2(b32, b64) < 2e-6
    assert cpu_ref.last_oob() == 0


def test_bp_is_fp_transpose_without_edge_rays():
    # half-integer rhozero: no ray runs along a pixel edge, and the reference's
    # backprojector is exactly the adjoint of its forward projector
    g = phantom.geometry(16, 13, numrhos=24)
    assert g.rhozero == -11.5
    A = F.fp_matrix(g.angles, g.rhozero, g.deltarho, g.numrhos, 16)
    B = F.bp_matrix(g.angles, g.rhozero, g.deltarho, g.numrhos, 16)
    assert abs(A - B.T).max() < 1e-12


def test_edge_rays_are_where_fp_and_bp_differ():
    # integer rhozero and theta = 0: vertical rays on pixel edges.  The
    # reference's forward projector gives them to the pixel right of the edge
    # (floor, forwardprojection.fut:35), its backprojector to neither side
    # (intersect_fact returns 0, backprojection.fut:30).
    ang = np.array([0.0], np.float32)
    A = F.fp_matrix(ang, -11.0, 1.0, 23, 16).toarray()
    B = F.bp_matrix(ang, -11.0, 1.0, 23, 16).toarray()
    ray = 11 + 3  # rho = 3: the edge between columns 10 and 11
    assert A[ray].sum() == pytest.approx(16.0)
    assert np.all(A[ray].reshape(16, 16)[:, 11] == 1.0)
    assert B[:, ray].sum() == 0.0


def test_sirt_fp32_restatement_close_to_fp64():
    size, a = 32, 24
    g = phantom.geometry(size, a, numrhos=46)
    img = phantom.ellipse_phantom(size, seed=1)
    ops = F.SirtOperators(g.angles, g.rhozero, g.deltarho, g.numrhos, size)
    b = (ops.A @ img.astype(np.float64)).astype(np.float32)
    res = []
    x64 = ops.iterate(np.zeros(size * size, np.float32), b, 30, res)
    x32 = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(size * size, np.float32), b, 30)
    assert rel_l2(x32, x64) < 1e-5
    assert res[-1] < res[0]


def test_sirt3d_oracles_agree():
    size, a = 8, 6
    g = phantom.geometry(size, a, numrhos=12)
    rhos = (g.rhozero + np.arange(12) * g.deltarho).astype(np.float32)
    proj = np.random.default_rng(0).random(size * a * 12).astype(np.float32)
    x64 = F.sirt3d(g.angles, rhos, proj, 5, size)
    x32 = cpu_ref.sirt3d(g.angles, rhos, proj, 5, size)
    assert x64.shape == (size ** 3,)
    assert rel_l2(x32, x64) < 1e-5


def test_cpu_sirt_rejects_odd_sides():
    """SIRT.fut:38-39 adds a (2*halfsize)^2 backprojection to the n-pixel image,
    so only even square sides are valid; the C restatement refuses the rest
    (the product's C-ABI answers SYNK_EINVAL for them)."""
    g = phantom.geometry(9, 6)
    sino = np.zeros(6 * g.numrhos, np.float32)
    with pytest.raises(ValueError):
        cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(81, np.float32), sino, 2)
    with pytest.raises(ValueError):
        cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(80, np.float32), sino, 2)
    rhos = np.float32(g.rhozero) + np.arange(g.numrhos, dtype=np.float32)
    with pytest.raises(ValueError):
        cpu_ref.sirt3d(g.angles, rhos, np.zeros(9 * sino.size, np.float32), 2, 9)


@pytest.mark.parametrize("size,a,nr", [(32, 20, None), (40, 33, 61)])
def test_fp64_backprojection_rows_match_the_matrix(size, a, nr):
    """The row-by-row FP64 backprojection (used where the full matrix would be
    too large) is the matrix oracle restricted to those rows."""
    g = phantom.geometry(size, a, numrhos=nr)
    y = np.random.default_rng(1).random(g.n_rays).astype(np.float32)
    full = F.backprojection(g.angles, g.rhozero, g.deltarho, size, y).reshape(size, size)
    rows = [0, 3, size // 2, size - 1]
    np.testing.assert_array_equal(F.backprojection_rows(g.angles, g.rhozero, g.deltarho, size, y, rows), full[rows])
