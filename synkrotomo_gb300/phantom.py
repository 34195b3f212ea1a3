"""Seeded synthetic phantoms and geometries for the parallel-beam workloads.

The reference's own datasets (``data/tooth.in``, ``fpinputf32rad*`` except
N=512, ``sirt3Dinputf32rad*``) are not shipped, so every workload here is a
seeded random-ellipse phantom with the shapes, sizes and value ranges that the
benchmark configurations name.  Pixel (row, col) of an N x N image covers
``[x, x+1) x [y, y+1)`` with ``x = col - N/2`` and ``y = row - N/2``, the
convention of futhark/forwardprojection.fut:22-51.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Geometry:
    """One 2D parallel-beam geometry in the reference's argument terms."""

    size: int            # image is size x size
    angles: np.ndarray   # float32 [a]
    numrhos: int         # detectors per angle
    rhozero: float       # rho of detector 0
    deltarho: float      # detector spacing

    @property
    def n_angles(self) -> int:
        return int(self.angles.size)

    @property
    def n_rays(self) -> int:
        return self.n_angles * self.numrhos


def default_detectors(size: int) -> int:
    """ceil(N*sqrt(2)): the detector count of the reference's datasets."""
    return int(math.ceil(size * math.sqrt(2.0)))


def geometry(size: int, n_angles: int, numrhos: int | None = None, deltarho: float = 1.0,
             arc: float = math.pi) -> Geometry:
    """Angles uniform in [0, arc) (float32), rhozero = -(numrhos-1)/2 * deltarho."""
    if numrhos is None:
        numrhos = default_detectors(size)
    angles = np.linspace(0.0, arc, n_angles, endpoint=False).astype(np.float32)
    rhozero = float(np.float32(-(numrhos - 1) / 2.0 * deltarho))
    return Geometry(int(size), angles, int(numrhos), rhozero, float(np.float32(deltarho)))


def ellipse_phantom(size: int, seed: int, n_ellipses: int = 10, centre_range: float = 0.6,
                    axis_range=(0.05, 0.4)) -> np.ndarray:
    """Random-ellipse phantom, float32 [size*size] row-major.

    Centres U[-c, c]*N/2, semi-axes U[lo, hi]*N/2, rotation U[0, pi),
    additive intensity U[0, 1]; a pixel belongs to an ellipse when its centre
    does.
    """
    rng = np.random.default_rng(seed)
    half = size / 2.0
    coords = np.arange(size, dtype=np.float64) - half + 0.5
    y, x = np.meshgrid(coords, coords, indexing="ij")
    img = np.zeros((size, size), np.float64)
    for _ in range(n_ellipses):
        cx, cy = rng.uniform(-centre_range, centre_range, 2) * half
        ax, ay = rng.uniform(axis_range[0], axis_range[1], 2) * half
        phi = rng.uniform(0.0, math.pi)
        val = rng.uniform(0.0, 1.0)
        c, s = math.cos(phi), math.sin(phi)
        u = (x - cx) * c + (y - cy) * s
        v = -(x - cx) * s + (y - cy) * c
        img[(u / ax) ** 2 + (v / ay) ** 2 <= 1.0] += val
    return img.astype(np.float32).ravel()


def ellipsoid_volume(size: int, n_slices: int, seed: int, n_ellipsoids: int = 12) -> np.ndarray:
    """Random 3D ellipsoid phantom, float32 [n_slices, size*size] (slice-major)."""
    rng = np.random.default_rng(seed)
    half = size / 2.0
    zh = n_slices / 2.0
    coords = np.arange(size, dtype=np.float64) - half + 0.5
    y, x = np.meshgrid(coords, coords, indexing="ij")
    vol = np.zeros((n_slices, size, size), np.float32)
    params = []
    for _ in range(n_ellipsoids):
        cx, cy = rng.uniform(-0.6, 0.6, 2) * half
        cz = rng.uniform(-0.6, 0.6) * zh
        ax, ay = rng.uniform(0.05, 0.4, 2) * half
        az = rng.uniform(0.05, 0.4) * zh
        phi = rng.uniform(0.0, math.pi)
        val = rng.uniform(0.0, 1.0)
        params.append((cx, cy, cz, ax, ay, az, math.cos(phi), math.sin(phi), val))
    for z in range(n_slices):
        zc = z - zh + 0.5
        sl = np.zeros((size, size), np.float64)
        for cx, cy, cz, ax, ay, az, c, s, val in params:
            dz = ((zc - cz) / az) ** 2
            if dz > 1.0:
                continue
            u = (x - cx) * c + (y - cy) * s
            v = -(x - cx) * s + (y - cy) * c
            sl[(u / ax) ** 2 + (v / ay) ** 2 <= 1.0 - dz] += val
        vol[z] = sl
    return vol.reshape(n_slices, size * size)


def add_noise(sino: np.ndarray, seed: int, rel_sigma: float = 0.01) -> np.ndarray:
    """Gaussian noise of sigma = rel_sigma * max(sino), float32."""
    rng = np.random.default_rng(seed + 7919)
    sino = np.asarray(sino, dtype=np.float32)
    sigma = rel_sigma * float(np.max(sino)) if sino.size else 0.0
    return (sino + rng.normal(0.0, sigma, sino.shape)).astype(np.float32)
