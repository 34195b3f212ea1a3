"""Writes tests/golden/oracle_small.npz: seeded small inputs of the projection
and SIRT programs with the outputs of both oracles.

The reference ships no expected outputs for its programs (its own pins are the
known-answer tests of archive/line_lib.fut and archive/projection_lib.fut,
checked in test_oracle_kats.py).  These fixtures freeze what the pinned
oracles give on a few seeded cases, inputs included, so that the GPU tests
compare against committed numbers and a change of the oracles shows up as a
failing CPU test.

Cases (name -> geometry):
  fp_*/bp_*: N, angles over [0, pi), detectors, deltarho
  sirt_*:    the same plus iterations, from a zero start

Run from the repository root: python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import cpu_ref  # noqa: E402
from oracle import fut_ref as F  # noqa: E402
from synkrotomo_gb300 import phantom  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_small.npz")

# (name, N, angles, detectors (None: ceil(N*sqrt(2))), deltarho)
PROJ_CASES = [
    ("a", 32, 30, None, 1.0),       # integer rhozero: rays along pixel edges at theta = 0, pi/2
    ("b", 64, 45, 92, 1.0),         # half-integer rhozero
    ("c", 40, 36, None, 0.5),       # three detectors per pixel
    ("d", 48, 40, 30, 1.0),         # detector row narrower than the image
]
# (name, N, angles, detectors, iterations, noise)
SIRT_CASES = [
    ("a", 32, 30, None, 20, 0.0),
    ("b", 64, 60, 92, 15, 0.01),
]


def cases():
    out = {}
    for name, n, a, nr, dr in PROJ_CASES:
        g = phantom.geometry(n, a, numrhos=nr, deltarho=dr)
        img = phantom.ellipse_phantom(n, seed=100 + n)
        y = np.random.default_rng(200 + n).random(g.n_rays).astype(np.float32)
        p = f"proj_{name}_"
        out[p + "geom"] = np.array([n, a, g.numrhos, g.rhozero, g.deltarho], np.float64)
        out[p + "angles"] = g.angles
        out[p + "image"] = img
        out[p + "sino"] = y
        out[p + "fp32"] = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
        out[p + "fp64"] = F.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
        out[p + "bp32"] = cpu_ref.backprojection(g.angles, g.rhozero, g.deltarho, n, y)
        out[p + "bp64"] = F.backprojection(g.angles, g.rhozero, g.deltarho, n, y)
    for name, n, a, nr, its, noise in SIRT_CASES:
        g = phantom.geometry(n, a, numrhos=nr)
        img = phantom.ellipse_phantom(n, seed=300 + n)
        b = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
        if noise:
            b = phantom.add_noise(b, 7, noise)
        x0 = np.zeros(n * n, np.float32)
        p = f"sirt_{name}_"
        out[p + "geom"] = np.array([n, a, g.numrhos, g.rhozero, g.deltarho, its], np.float64)
        out[p + "angles"] = g.angles
        out[p + "sino"] = b.astype(np.float32)
        out[p + "x32"] = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, x0, b, its)
        out[p + "x64"] = F.SirtOperators(g.angles, g.rhozero, g.deltarho, g.numrhos, n).iterate(x0, b, its)
    return out


def main():
    np.savez_compressed(OUT, **cases())
    print("wrote", OUT)


if __name__ == "__main__":
    main()
