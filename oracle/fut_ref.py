"""FP64 NumPy restatement of synkrotomo's parallel-beam projection + SIRT path.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): this module is the
checker, never the thing measured or shipped.

Every function restates one piece of the reference's Futhark code, cited as
``file:line`` relative to the reference project root.  The arithmetic is done
in FP64 on the float32 inputs ("the reference math, evaluated exactly"), while
the control flow (steep/flat split, the transposed traversal of flat lines, the
floor/ceil decisions, the bounds tests) follows the reference step by step.

Geometry convention of the reference (``futhark/forwardprojection.fut:26-29``,
``futhark/sirtlib.fut:41``): the ray of angle theta and detector r is the line
``rho = x*cos(theta) - y*sin(theta)`` with ``rho = rhozero + r*deltarho``;
``x = column - N/2`` and ``y = row - N/2`` for the row-major image, pixel
(row, col) being the unit square ``[x, x+1) x [y, y+1)``.

The projectors are returned as SciPy sparse matrices built from the
reference's per-ray (FP) and per-pixel (BP) rules, so SIRT runs as sparse
mat-vecs and finishes in seconds at the test sizes.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

# backprojection.fut:20  (fact = sqrt(2)/2)
FACT = math.sqrt(2.0) / 2.0


# ---------------------------------------------------------------------------
# sirtlib  (futhark/sirtlib.fut)
# ---------------------------------------------------------------------------

def is_flat(cos, sin):
    """sirtlib.fut:6-7: a line is flat when |sin| >= |cos|."""
    return np.abs(sin) >= np.abs(cos)


def safe_inverse(v):
    """sirtlib.fut:9-13: 1/v elementwise with 0 -> 0."""
    v = np.asarray(v, dtype=np.float64)
    out = np.zeros_like(v)
    nz = v != 0.0
    out[nz] = 1.0 / v[nz]
    return out


def preprocess(angles):
    """sirtlib.fut:28-44, per original angle index.

    Returns ``(cost, sint, lbase, flat)`` where (cost, sint, lbase) is the
    reference's line triple: ``(cos, -sin, sqrt(1+(sin/cos)^2))`` for steep
    angles and ``(-sin, cos, sqrt(1+(cos/sin)^2))`` for flat ones, the latter
    describing the line in the transposed image (sirtlib.fut:41).  The
    reference also partitions the angles steep-first (sirtlib.fut:39, 42-43);
    that order only permutes rows of the sinogram and is undone at the API
    (sirtlib.fut:24-25), so it is kept implicit here.
    """
    th = np.asarray(angles, dtype=np.float32).astype(np.float64)
    cos = np.cos(th)
    sin = np.sin(th)
    flat = is_flat(cos, sin)
    with np.errstate(divide="ignore", invalid="ignore"):
        lsteep = np.sqrt(1.0 + (sin / cos) ** 2)
        lflat = np.sqrt(1.0 + (cos / sin) ** 2)
    cost = np.where(flat, -sin, cos)
    sint = np.where(flat, cos, -sin)
    lbase = np.where(flat, lflat, lsteep)
    return cost, sint, lbase, flat


# ---------------------------------------------------------------------------
# forward projection  (futhark/forwardprojection.fut)
# ---------------------------------------------------------------------------

def _fp_rows(cost, sint, lbase, rho, halfsize):
    """forwardprojection.fut:26-56 for one line and a vector of rhos.

    Returns (ray, row, col, weight) entries in the frame of the traversed
    image (the transposed image for flat lines), skipping out-of-bounds
    pixels exactly as the reference's bounds flags do (lines 43-44, 53-54).
    """
    slope = -sint / cost                                  # line 26
    intercept = rho / cost                                # line 29
    i = np.arange(-halfsize, halfsize, dtype=np.float64)  # line 57
    xbot = i[None, :] * slope + intercept[:, None]        # line 32
    xtop = xbot + slope                                   # line 33
    xpixbot = np.floor(xbot)                              # line 35
    xpixtop = np.floor(xtop)                              # line 36
    xpixmax = np.maximum(xpixbot, xpixtop)                # line 38
    xdiff = xtop - xbot                                   # line 40
    single = xpixbot == xpixtop                           # line 42
    botin = (xpixbot >= -halfsize) & (xpixbot < halfsize)            # line 43
    topin = (~single) & (xpixtop >= -halfsize) & (xpixtop < halfsize)  # line 44
    with np.errstate(divide="ignore", invalid="ignore"):
        lxbot = np.where(single, lbase, (xpixmax - xbot) / xdiff * lbase)  # 46-47
        lxtop = (xtop - xpixmax) / xdiff * lbase                           # 48
    ray = np.broadcast_to(np.arange(rho.size)[:, None], xbot.shape)
    row = np.broadcast_to((i + halfsize).astype(np.int64)[None, :], xbot.shape)
    out = []
    for inb, xp, w in ((botin, xpixbot, lxbot), (topin, xpixtop, lxtop)):
        col = (xp + halfsize).astype(np.int64)
        out.append((ray[inb], row[inb], col[inb], w[inb]))
    return out


def fp_matrix(angles, rhozero, deltarho, numrhos, size):
    """System matrix of the reference forward projector as CSR (rays x pixels).

    Rows are angle-major rays ``k*numrhos + r`` (the output order of
    forwardprojection.fut:65 / sirtlib.fut:24-25); columns are row-major
    pixels of the ``size x size`` image.  Flat lines traverse the transposed
    image (forwardprojection.fut:80-82, 63), so their (row, col) are swapped
    back here.
    """
    halfsize = int(size) // 2
    cost, sint, lbase, flat = preprocess(angles)
    rhos = float(np.float32(rhozero)) + np.arange(numrhos, dtype=np.float64) * float(np.float32(deltarho))
    rows, cols, vals = [], [], []
    for k in range(cost.size):
        for ray, row, col, w in _fp_rows(cost[k], sint[k], lbase[k], rhos, halfsize):
            if flat[k]:
                row, col = col, row
            rows.append(k * numrhos + ray)
            cols.append(row * size + col)
            vals.append(w)
    m = sp.coo_matrix(
        (np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
        shape=(cost.size * numrhos, size * size),
    )
    return m.tocsr()


def forwardprojection(angles, rhozero, deltarho, numrhos, image):
    """forwardprojection.fut:71-84 ``main``: angle-major sinogram [a*numrhos]."""
    image = np.asarray(image, dtype=np.float32)
    size = int(math.isqrt(image.size))                    # line 76
    a = fp_matrix(angles, rhozero, deltarho, numrhos, size)
    return a @ image.astype(np.float64)


# ---------------------------------------------------------------------------
# backprojection  (futhark/backprojection.fut)
# ---------------------------------------------------------------------------

def intersect_fact(plus, minus, mini, maxi):
    """backprojection.fut:22-33: overlap of [minus, plus] with [mini, maxi]
    as a fraction of plus-minus, 0 when there is no overlap, capped at 1."""
    lo = np.maximum(plus - mini, 0.0)
    hi = np.maximum(maxi - minus, 0.0)
    diff = plus - minus
    inside = np.minimum(lo, hi)
    with np.errstate(divide="ignore", invalid="ignore"):
        prop = np.where(inside == 0.0, 0.0, inside / diff)
    return np.minimum(prop, 1.0)


def first_detector(cost, sint, xmin, ymin, rhozero, deltarho):
    """backprojection.fut:50-53: index s of the first detector whose ray can
    touch the pixel with lower-left corner (xmin, ymin) for the line normal
    (cost, sint): ``ceil((rho(centre - fact*normal) - rhozero)/deltarho)``."""
    x = xmin + 0.5 - FACT * cost
    y = ymin + 0.5 - FACT * sint
    rho = cost * x + sint * y
    return np.ceil((rho - rhozero) / deltarho)


def bp_weight(cost, sint, lbase, xmin, ymin, sprime, rhozero, deltarho):
    """backprojection.fut:49, 54-62: intersection length of detector sprime's
    ray with the pixel (xmin, ymin) in the line's own (possibly transposed)
    frame."""
    slope = -sint / cost
    xbase = ymin * slope
    r = sprime * deltarho + rhozero
    xbot = xbase + r / cost
    xtop = xbot + slope
    return intersect_fact(np.maximum(xbot, xtop), np.minimum(xbot, xtop), xmin, xmin + 1.0) * lbase


def rhos_per_pixel(deltarho):
    """backprojection.fut:87: ceil(sqrt(2)/deltarho), evaluated in float32 as
    the reference does."""
    return int(np.ceil(np.float32(np.sqrt(np.float32(2.0))) / np.float32(deltarho)))


def bp_matrix(angles, rhozero, deltarho, numrhos, size, count_oob=False):
    """System matrix of the reference backprojector as CSR (pixels x rays).

    For every pixel and line, the reference sums ``rhosprpixel`` detectors
    starting at ``first_detector`` (backprojection.fut:48-65) and reads the
    sinogram unchecked (line 64).  Here a detector outside [0, numrhos) adds
    nothing; with ``count_oob`` the number of such reads that carry a
    non-zero weight is returned as well (0 whenever the reference's own read
    stays inside the ray's row).
    """
    halfsize = int(size) // 2
    rz = float(np.float32(rhozero))
    dr = float(np.float32(deltarho))
    rpp = rhos_per_pixel(deltarho)
    cost, sint, lbase, flat = preprocess(angles)
    coords = np.arange(-halfsize, halfsize, dtype=np.float64)
    ymin, xmin = np.meshgrid(coords, coords, indexing="ij")  # irow, icolumn (line 44-46)
    rows, cols, vals = [], [], []
    oob = 0
    for k in range(cost.size):
        s = first_detector(cost[k], sint[k], xmin, ymin, rz, dr)
        for i in range(rpp):
            sprime = s + i
            w = bp_weight(cost[k], sint[k], lbase[k], xmin, ymin, sprime, rz, dr)
            det = sprime.astype(np.int64)
            ok = (det >= 0) & (det < numrhos)
            oob += int(np.count_nonzero((~ok) & (w != 0.0)))
            keep = ok & (w != 0.0)
            irow = (ymin[keep] + halfsize).astype(np.int64)
            icol = (xmin[keep] + halfsize).astype(np.int64)
            if flat[k]:
                # bp_flat is computed in the transposed frame and transposed back (75-78)
                pix = icol * size + irow
            else:
                pix = irow * size + icol
            rows.append(pix)
            cols.append(k * numrhos + det[keep])
            vals.append(w[keep])
    m = sp.coo_matrix(
        (np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
        shape=(size * size, cost.size * numrhos),
    ).tocsr()
    return (m, oob) if count_oob else m


def backprojection_rows(angles, rhozero, deltarho, size, projections, rows):
    """Rows ``rows`` of backprojection.fut:82-93 ``main`` ([len(rows), size]),
    from the same per-pixel rule as ``bp_matrix`` without building the matrix:
    for a steep line an image row is a frame row; a flat line works in the
    transposed frame (lines 75-78), where the image row is a frame column."""
    halfsize = int(size) // 2
    rz = float(np.float32(rhozero))
    dr = float(np.float32(deltarho))
    rpp = rhos_per_pixel(deltarho)
    proj = np.asarray(projections, dtype=np.float32).astype(np.float64)
    a = np.asarray(angles).size
    numrhos = proj.size // a
    cost, sint, lbase, flat = preprocess(angles)
    rows = np.asarray(rows, dtype=np.int64)
    coords = np.arange(-halfsize, halfsize, dtype=np.float64)
    fixed = rows.astype(np.float64)[:, None] - halfsize          # [R, 1]
    out = np.zeros((rows.size, int(size)))
    for k in range(cost.size):
        if flat[k]:
            xmin, ymin = np.broadcast_to(fixed, out.shape), np.broadcast_to(coords[None, :], out.shape)
        else:
            ymin, xmin = np.broadcast_to(fixed, out.shape), np.broadcast_to(coords[None, :], out.shape)
        s = first_detector(cost[k], sint[k], xmin, ymin, rz, dr)
        for i in range(rpp):
            sprime = s + i
            w = bp_weight(cost[k], sint[k], lbase[k], xmin, ymin, sprime, rz, dr)
            det = sprime.astype(np.int64)
            ok = (det >= 0) & (det < numrhos) & (w != 0.0)
            out += np.where(ok, w * proj[k * numrhos + np.clip(det, 0, numrhos - 1)], 0.0)
    return out


def backprojection(angles, rhozero, deltarho, size, projections):
    """backprojection.fut:82-93 ``main``: image [size*size]."""
    projections = np.asarray(projections, dtype=np.float32)
    a = np.asarray(angles).size
    numrhos = projections.size // a                        # line 89
    b = bp_matrix(angles, rhozero, deltarho, numrhos, int(size))
    return b @ projections.astype(np.float64)


# ---------------------------------------------------------------------------
# SIRT  (futhark/SIRT.fut, futhark/SIRT3D.fut)
# ---------------------------------------------------------------------------

class SirtOperators:
    """The matrices and normalisers of one SIRT geometry (SIRT.fut:15-25)."""

    def __init__(self, angles, rhozero, deltarho, numrhos, size):
        self.A = fp_matrix(angles, rhozero, deltarho, numrhos, size)
        self.B = bp_matrix(angles, rhozero, deltarho, numrhos, size)
        n = size * size
        self.R = safe_inverse(self.A @ np.ones(n))                 # lines 22-23
        self.C = safe_inverse(self.B @ np.ones(self.A.shape[0]))   # line 25

    def iterate(self, image, projections, iterations, residuals=None):
        """SIRT.fut:27-39: x <- x + C*BP(R*(b - FP(x))), ``iterations`` times.

        When ``residuals`` is a list, ||FP(x_k) - b|| / ||b|| is appended for
        every iterate x_0 .. x_iterations.
        """
        x = np.asarray(image, dtype=np.float32).astype(np.float64).copy()
        b = np.asarray(projections, dtype=np.float32).astype(np.float64)
        bn = np.linalg.norm(b)
        for _ in range(int(iterations)):
            e = b - self.A @ x
            if residuals is not None:
                residuals.append(np.linalg.norm(e) / bn if bn else 0.0)
            x += self.C * (self.B @ (self.R * e))
        if residuals is not None:
            e = b - self.A @ x
            residuals.append(np.linalg.norm(e) / bn if bn else 0.0)
        return x


def sirt(angles, rhozero, deltarho, image, projections, iterations, residuals=None):
    """SIRT.fut:43-49 ``main``: reconstruct from ``image`` (the start)."""
    image = np.asarray(image, dtype=np.float32)
    size = int(math.isqrt(image.size))                    # line 16
    a = np.asarray(angles).size
    numrhos = np.asarray(projections).size // a           # line 18
    ops = SirtOperators(angles, rhozero, deltarho, numrhos, size)
    return ops.iterate(image, projections, iterations, residuals)


def sirt3d(angles, rhos, projections, iterations, size):
    """SIRT3D.fut:18-29 (intended semantics): ``size`` independent slices,
    zero start, slice i reads ``projections[i*r*a:(i+1)*r*a]``.

    The reference passes ``rhos`` where SIRT expects (rhozero, deltarho)
    (SIRT3D.fut:27 vs SIRT.fut:9-14); the convention of
    archive/projection_lib.fut:114-115 is used: rhozero = rhos[0],
    deltarho = rhos[1] - rhos[0].
    """
    rhos = np.asarray(rhos, dtype=np.float32)
    a = np.asarray(angles).size
    r = rhos.size
    rhozero = float(rhos[0])
    deltarho = float(np.float32(rhos[1] - rhos[0])) if r > 1 else 1.0
    ops = SirtOperators(angles, rhozero, deltarho, r, int(size))
    proj = np.asarray(projections, dtype=np.float32)
    out = []
    for i in range(int(size)):
        out.append(ops.iterate(np.zeros(size * size, np.float32), proj[i * r * a:(i + 1) * r * a], iterations))
    return np.concatenate(out)


def relative_residual(A, x, b):
    """||A x - b||_2 / ||b||_2 in FP64."""
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(A @ np.asarray(x, np.float64) - b) / np.linalg.norm(b))


# --- validation programs (futhark/tools/*.fut) --------------------------------
# std_dev = 0.05f32 in all three programs (diff.fut:2, sanityCheck.fut:2)
TOOLS_STD_DEV = np.float32(0.05)


def tools_diff(sane, test):
    """tools/diff.fut:4-6: indices where |s - t| > std_dev get i, the others -1;
    filter (> 0) keeps the positive ones, so index 0 is never counted."""
    s = np.asarray(sane, np.float32)
    t = np.asarray(test, np.float32)
    d = np.abs(s - t)                          # f32 arithmetic, as the program
    marks = np.where(d > TOOLS_STD_DEV, np.arange(s.size), -1)
    return np.int32(np.count_nonzero(marks > 0))


def tools_mse(sane, test):
    """tools/mse.fut:2-3: sum of (s - t)**2 divided by n (evaluated in FP64)."""
    s = np.asarray(sane, np.float64)
    t = np.asarray(test, np.float64)
    return float(np.sum((s - t) ** 2) / s.size)


def tools_sanity(sane, test):
    """tools/sanityCheck.fut:3-4: every |s - t| < std_dev."""
    s = np.asarray(sane, np.float32)
    t = np.asarray(test, np.float32)
    return bool(np.all(np.abs(s - t) < TOOLS_STD_DEV))
