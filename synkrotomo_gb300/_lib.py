"""ctypes binding of libsynk.so (the C ABI declared in include/synk.h).

The library is the only compute path: there is no CPU fallback.  Loading
fails with a RuntimeError when libsynk.so has not been built.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_lib = None

c_f32p = ctypes.POINTER(ctypes.c_float)
c_f64p = ctypes.POINTER(ctypes.c_double)
c_i32p = ctypes.POINTER(ctypes.c_int32)
c_ctx = ctypes.c_void_p

SYNK_OK = 0
SYNK_EINVAL = 1
SYNK_ECUDA = 2
SYNK_ETIMEOUT = 3
SYNK_ENOMEM = 4


class SynkOptions(ctypes.Structure):
    """``synk_sirt_options`` of include/synk.h."""

    _fields_ = [
        ("tol", ctypes.c_double),
        ("residuals", ctypes.c_void_p),
        ("iterations_done", ctypes.c_void_p),
        ("fp_split", ctypes.c_int32),
        ("bp_split", ctypes.c_int32),
        ("grid_blocks", ctypes.c_int32),
    ]


class SynkProblem(ctypes.Structure):
    """``synk_sirt_problem`` of include/synk.h."""

    _fields_ = [
        ("angles", ctypes.c_void_p),
        ("a", ctypes.c_int64),
        ("rhozero", ctypes.c_float),
        ("deltarho", ctypes.c_float),
        ("numrhos", ctypes.c_int32),
        ("size", ctypes.c_int32),
        ("nslices", ctypes.c_int32),
        ("iterations", ctypes.c_int32),
        ("image", ctypes.c_void_p),
        ("projections", ctypes.c_void_p),
        ("out", ctypes.c_void_p),
        ("residuals", ctypes.c_void_p),
        ("iterations_done", ctypes.c_void_p),
        ("fp_split", ctypes.c_int32),
        ("bp_split", ctypes.c_int32),
    ]


# name -> (restype, argtypes); kept in the order of include/synk.h
SIGNATURES = {
    "synk_context_new": (ctypes.c_int, [ctypes.POINTER(c_ctx), ctypes.c_int, ctypes.c_void_p]),
    "synk_context_free": (None, [c_ctx]),
    "synk_context_set_stream": (ctypes.c_int, [c_ctx, ctypes.c_void_p]),
    "synk_context_sync": (ctypes.c_int, [c_ctx]),
    "synk_context_set_barrier_limit": (ctypes.c_int, [c_ctx, ctypes.c_uint64, ctypes.c_int32]),
    "synk_context_get_error": (ctypes.c_char_p, [c_ctx]),
    "synk_version": (ctypes.c_char_p, []),
    "synk_forwardprojection": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64]),
    "synk_forwardprojection_sparse": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                     ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p,
                                                     ctypes.c_int64]),
    "synk_backprojection": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64]),
    "synk_backprojection_sparse": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                  ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p,
                                                  ctypes.c_int64]),
    "synk_SIRT": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float,
                                 ctypes.c_float, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                 ctypes.c_int32]),
    "synk_SIRT3D": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                   ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32]),
    "synk_sirt_slices": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                        ctypes.POINTER(SynkOptions)]),
    "synk_sirt_resident_blocks": (ctypes.c_int, []),
    "synk_sirt_batch": (ctypes.c_int, [c_ctx, ctypes.c_int32, ctypes.POINTER(SynkProblem), ctypes.c_double,
                                       ctypes.c_int32]),
    "synk_sirt_plan_new": (ctypes.c_int, [c_ctx, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32,
                                          ctypes.POINTER(SynkProblem), ctypes.c_double, ctypes.c_int32]),
    "synk_sirt_plan_launch": (ctypes.c_int, [c_ctx, ctypes.c_void_p]),
    "synk_sirt_plan_free": (None, [ctypes.c_void_p]),
    "synk_csr_new": (ctypes.c_int, [c_ctx, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_int32]),
    "synk_csr_free": (None, [ctypes.c_void_p]),
    "synk_csr_shape": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "synk_csr_arrays": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p),
                                       ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p)]),
    "synk_csr_spmv": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "synk_csr_spmv_t": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "synk_spmv_csr32": (ctypes.c_int, [c_ctx, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p]),
    "synk_gemm_bf16": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_int32]),
    "synk_conv3x3_bf16": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                         ctypes.c_int32]),
    "synk_conv3x3_wgrad_bf16": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                               ctypes.c_int32, ctypes.c_int32]),
    "synk_unet_new": (ctypes.c_int, [c_ctx, ctypes.POINTER(ctypes.c_void_p), ctypes.c_int32, ctypes.c_int32,
                                     ctypes.c_uint64]),
    "synk_unet_free": (None, [ctypes.c_void_p]),
    "synk_unet_num_params": (ctypes.c_int64, [ctypes.c_void_p]),
    "synk_unet_params": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "synk_unet_optimizer_state": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.POINTER(ctypes.c_int64), ctypes.c_int32]),
    "synk_unet_forward": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "synk_unet_train_step": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                            ctypes.c_float, ctypes.c_int32, ctypes.c_void_p]),
    "synk_unet_gradients": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p]),
    "synk_compare": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_float]),
    "synk_diff": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "synk_mse": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "synk_sanityCheck": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "synk_backprojection_noalloc": (ctypes.c_int, [c_ctx, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                                   ctypes.c_float, ctypes.c_float, ctypes.c_int32, ctypes.c_void_p,
                                                   ctypes.c_int64]),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libsynk.so and declare the signatures of include/synk.h."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise RuntimeError(
                f"libsynk.so not found at {path}: build it first "
                "(python -c 'import __graft_entry__ as g; g.build()' or python -m synkrotomo_gb300.build)")
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L
