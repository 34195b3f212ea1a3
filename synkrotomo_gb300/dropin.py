"""Classes behind the ``futhark`` drop-in package.

The reference's Python surface is generated by ``futhark pyopencl --library``
(Makefile:1-4): one module per program, one class named after the module,
an ``entry_points`` table and a ``main(*args)`` method returning a device
array that callers ``.get()`` (README.md:21-25).  These classes keep those
names, the argument order, the float32 / int32 argument types and the
flattened layouts, and run on libsynk instead of OpenCL.
"""
from __future__ import annotations

import math
import warnings

import numpy as np
import torch

from . import runtime as rt


class DetectorCoverageWarning(UserWarning):
    """The detector row is narrower than the image diagonal."""


def check_detector_coverage(numrhos: int, deltarho: float, size: int, program: str) -> bool:
    """Warn when the detector row (numrhos * deltarho) is narrower than the
    image diagonal, ceil(size * sqrt(2)).  A pixel's detector window can then
    leave the row: here such detectors contribute 0, where the reference reads
    the sinogram out of range (backprojection.fut:64).  Returns whether it
    warned; invalid arguments are left to the library's checks."""
    if size <= 0 or numrhos <= 0 or not deltarho > 0:
        return False
    need = math.ceil(size * math.sqrt(2.0))
    if numrhos * deltarho < need:
        warnings.warn(f"{program}: the detector row ({numrhos} detectors x {deltarho}) is narrower than the "
                      f"image diagonal (ceil({size}*sqrt(2)) = {need}); detectors outside it contribute 0 "
                      "(the reference reads out of range there)", DetectorCoverageWarning, stacklevel=3)
        return True
    return False


class _Entry:
    """Common constructor: the reference's keyword arguments (OpenCL platform
    and device preferences, group sizes) are accepted and ignored; ``device``
    selects the CUDA device."""

    entry_points: dict = {}

    def __init__(self, *args, device: int | None = None, **kwargs):
        if not torch.cuda.is_available():
            raise RuntimeError(f"{type(self).__name__}: a CUDA GPU is required (no CPU fallback exists)")
        self.device = torch.cuda.current_device() if device is None else int(device)
        rt.context(self.device)   # loads libsynk now: fail at construction, not at first call

    def _wrap(self, t: torch.Tensor) -> rt.DeviceArray:
        return rt.DeviceArray(t, rt.context(self.device))


class forwardprojection(_Entry):
    """futhark/forwardprojection.fut:71-84."""

    entry_points = {"main": (["[]f32", "f32", "f32", "i32", "[]f32"], ["[]f32"])}
    _sparse = False

    def main(self, angles, rhozero, deltarho, numrhos, image):
        with torch.cuda.device(self.device):
            a = rt.to_device_f32(angles, 0, "angles", self.device)
            rz = rt.scalar_f32(rhozero, 1, "rhozero")
            dr = rt.scalar_f32(deltarho, 2, "deltarho")
            nr = rt.scalar_i32(numrhos, 3, "numrhos")
            img = rt.to_device_f32(image, 4, "image", self.device)
            out = rt.forwardprojection(a, rz, dr, nr, img, sparse=self._sparse)
            return self._wrap(out)


class forwardprojection_sparse(forwardprojection):
    """futhark/forwardprojection_sparse.fut:26-40 (same program, sparse-view data)."""

    _sparse = True


class backprojection(_Entry):
    """futhark/backprojection.fut:82-93."""

    entry_points = {"main": (["[]f32", "f32", "f32", "i32", "[]f32"], ["[]f32"])}
    _sparse = False

    def main(self, angles, rhozero, deltarho, size, projections):
        with torch.cuda.device(self.device):
            a = rt.to_device_f32(angles, 0, "angles", self.device)
            rz = rt.scalar_f32(rhozero, 1, "rhozero")
            dr = rt.scalar_f32(deltarho, 2, "deltarho")
            sz = rt.scalar_i32(size, 3, "size")
            proj = rt.to_device_f32(projections, 4, "projections", self.device)
            if a.numel():
                check_detector_coverage(proj.numel() // a.numel(), dr, sz, type(self).__name__)
            out = rt.backprojection(a, rz, dr, sz, proj, sparse=self._sparse)
            return self._wrap(out)


class backprojection_sparse(backprojection):
    """futhark/backprojection_sparse.fut:26-37 (same program, sparse-view data)."""

    _sparse = True


class SIRT(_Entry):
    """futhark/SIRT.fut:43-49."""

    entry_points = {"main": (["[]f32", "f32", "f32", "*[]f32", "[]f32", "i32"], ["[]f32"])}

    def main(self, angles, rhozero, deltarho, image, projections, iterations):
        with torch.cuda.device(self.device):
            a = rt.to_device_f32(angles, 0, "angles", self.device)
            rz = rt.scalar_f32(rhozero, 1, "rhozero")
            dr = rt.scalar_f32(deltarho, 2, "deltarho")
            img = rt.to_device_f32(image, 3, "image", self.device)
            proj = rt.to_device_f32(projections, 4, "projections", self.device)
            its = rt.scalar_i32(iterations, 5, "iterations")
            if a.numel():
                check_detector_coverage(proj.numel() // a.numel(), dr, math.isqrt(img.numel()), "SIRT")
            out = rt.sirt(a, rz, dr, img, proj, its)
            return self._wrap(out)


class SIRT3D(_Entry):
    """futhark/SIRT3D.fut:18-29 (intended semantics: rhozero = rhos[0],
    deltarho = rhos[1] - rhos[0], ``size`` slices from a zero start).  The
    keyword ``nslices`` (no reference counterpart) reconstructs a stack of
    that many size x size slices instead of ``size``."""

    entry_points = {"main": (["[]f32", "[]f32", "[]f32", "i32", "i32"], ["[]f32"])}

    def main(self, angles, rhos, projections, iterations, size, nslices=None):
        with torch.cuda.device(self.device):
            a = rt.to_device_f32(angles, 0, "angles", self.device)
            rh = rt.to_device_f32(rhos, 1, "rhos", self.device)
            proj = rt.to_device_f32(projections, 2, "projections", self.device)
            its = rt.scalar_i32(iterations, 3, "iterations")
            sz = rt.scalar_i32(size, 4, "size")
            ns = None if nslices is None else rt.scalar_i32(nslices, 5, "nslices")
            out = rt.sirt3d(a, rh, proj, its, sz, nslices=ns)
            return self._wrap(out)


def _np(x):
    return np.asarray(x)


class _Compare(_Entry):
    """The reference's validation programs (futhark/tools/*.fut): main(sane, test)
    on two float32 arrays of one length, returning a scalar as Futhark's
    generated classes do for scalar results."""

    _program = ""

    def main(self, sane, test):
        with torch.cuda.device(self.device):
            s = rt.to_device_f32(sane, 0, "sane", self.device)
            t = rt.to_device_f32(test, 1, "test", self.device)
            if s.numel() != t.numel():
                raise ValueError(f"{self._program}: sane has {s.numel()} elements and test {t.numel()}")
            return rt.compare_program(self._program, s, t)


class diff(_Compare):
    """futhark/tools/diff.fut: the number of indices i > 0 with |sane-test| > 0.05 (i32)."""

    entry_points = {"main": (["[]f32", "[]f32"], ["i32"])}
    _program = "diff"


class mse(_Compare):
    """futhark/tools/mse.fut: the mean squared difference (f32)."""

    entry_points = {"main": (["[]f32", "[]f32"], ["f32"])}
    _program = "mse"


class sanityCheck(_Compare):
    """futhark/tools/sanityCheck.fut: whether every |sane-test| < 0.05 (bool)."""

    entry_points = {"main": (["[]f32", "[]f32"], ["bool"])}
    _program = "sanityCheck"
