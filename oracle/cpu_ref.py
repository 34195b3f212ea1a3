"""ctypes wrapper of the FP32 C restatement (``oracle/cpu_ref.c``).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libcpuref.so")
_TIMED_PATH = os.path.join(_HERE, "_build", "libcpuref_timed.so")
_libs = {}
_active = "parity"

_f32p = ctypes.POINTER(ctypes.c_float)


def build(force: bool = False) -> str:
    """Compile ``cpu_ref.c`` (parity and timed builds) with ``oracle/Makefile``."""
    src = os.path.join(_HERE, "cpu_ref.c")
    stale = any(not os.path.exists(p) or os.path.getmtime(p) < os.path.getmtime(src) for p in (_LIB_PATH, _TIMED_PATH))
    if force or stale:
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "all"], check=True)
    return _LIB_PATH


def use_build(kind: str) -> str:
    """Select the library the functions below call: "parity" (the default:
    float32 rounding as written, what the tests compare with) or "timed" (the
    same source tuned for the host CPU, what bench.py times).  Returns the
    previous selection."""
    global _active
    if kind not in ("parity", "timed"):
        raise ValueError(f"unknown cpu_ref build {kind!r}")
    prev, _active = _active, kind
    return prev


def lib():
    L = _libs.get(_active)
    if L is None:
        build()
        L = ctypes.CDLL(_LIB_PATH if _active == "parity" else _TIMED_PATH)
        L.cpuref_forwardprojection.argtypes = [_f32p, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                               _f32p, ctypes.c_int64, _f32p]
        L.cpuref_backprojection.argtypes = [_f32p, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int,
                                            _f32p, ctypes.c_int64, _f32p]
        L.cpuref_sirt.argtypes = [_f32p, ctypes.c_int, ctypes.c_float, ctypes.c_float, _f32p, ctypes.c_int64,
                                  _f32p, ctypes.c_int64, ctypes.c_int, _f32p]
        L.cpuref_sirt3d.argtypes = [_f32p, ctypes.c_int, _f32p, ctypes.c_int, _f32p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, _f32p]
        L.cpuref_last_oob.restype = ctypes.c_int64
        L.cpuref_set_threads.argtypes = [ctypes.c_int]
        _libs[_active] = L
    return L


def _p(a):
    return a.ctypes.data_as(_f32p)


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel())


def set_threads(n: int = 0) -> int:
    """Set the OpenMP thread count (0 keeps it); returns the count in use."""
    return int(lib().cpuref_set_threads(int(n)))


def forwardprojection(angles, rhozero, deltarho, numrhos, image):
    angles, image = _f32(angles), _f32(image)
    out = np.empty(angles.size * int(numrhos), np.float32)
    rc = lib().cpuref_forwardprojection(_p(angles), angles.size, float(rhozero), float(deltarho), int(numrhos),
                                        _p(image), image.size, _p(out))
    if rc:
        raise MemoryError("cpu_ref: allocation failed")
    return out


def backprojection(angles, rhozero, deltarho, size, projections):
    angles, projections = _f32(angles), _f32(projections)
    hs = int(size) // 2
    out = np.empty(4 * hs * hs, np.float32)
    rc = lib().cpuref_backprojection(_p(angles), angles.size, float(rhozero), float(deltarho), int(size),
                                     _p(projections), projections.size, _p(out))
    if rc:
        raise MemoryError("cpu_ref: allocation failed")
    return out


def _check_sirt(rc, n):
    if rc == 2:
        raise ValueError(f"SIRT needs an even square image side (got {n} pixels)")
    if rc:
        raise MemoryError("cpu_ref: allocation failed")


def sirt(angles, rhozero, deltarho, image, projections, iterations):
    angles, image, projections = _f32(angles), _f32(image), _f32(projections)
    out = np.empty(image.size, np.float32)
    rc = lib().cpuref_sirt(_p(angles), angles.size, float(rhozero), float(deltarho), _p(image), image.size,
                           _p(projections), projections.size, int(iterations), _p(out))
    _check_sirt(rc, image.size)
    return out


def sirt3d(angles, rhos, projections, iterations, size, nslices=None):
    angles, rhos, projections = _f32(angles), _f32(rhos), _f32(projections)
    ns = int(size) if nslices is None else int(nslices)
    out = np.empty(ns * int(size) * int(size), np.float32)
    rc = lib().cpuref_sirt3d(_p(angles), angles.size, _p(rhos), rhos.size, _p(projections), int(iterations),
                             int(size), ns, _p(out))
    _check_sirt(rc, int(size) ** 2)
    return out


def last_oob() -> int:
    return int(lib().cpuref_last_oob())
