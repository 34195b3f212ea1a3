"""Autotuner of the persistent SIRT kernel's launch shape.

Tunables per problem:
  fp_split     1/2/4/8 warps share one ray of the forward phase (rows split);
               8/fp_split detectors (x 32 angles) per block item
  bp_split     1/2/4/8 warps share one pixel strip of the backward phase
               (angles split); tiles of 32 x 4*8/bp_split pixels
  grid_blocks  blocks of the cooperative launch (all resident, or half), or
               -1: the phase-split engine (one launch per phase and iteration)
Each candidate is timed on the problem itself (a few iterations, CUDA events);
the winner is cached in a JSON file keyed by the size bucket
(image side, angle count, detector count, slices rounded to powers of two), so
a bucket is measured once per machine.  Cache file: $SYNK_TUNE_CACHE, else
~/.cache/synkrotomo_gb300/autotune.json.
"""
from __future__ import annotations

import itertools
import json
import math
import os
import threading

_lock = threading.Lock()
SPLITS = (1, 2, 4, 8)


def cache_path() -> str:
    p = os.environ.get("SYNK_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "synkrotomo_gb300", "autotune.json")


def _pow2_bucket(v: int) -> int:
    return 1 << max(0, int(math.ceil(math.log2(max(1, int(v))))))


def bucket(size: int, n_angles: int, numrhos: int, nslices: int = 1) -> str:
    return f"N{_pow2_bucket(size)}_a{_pow2_bucket(n_angles)}_d{_pow2_bucket(numrhos)}_s{_pow2_bucket(nslices)}"


def load_cache(path: str | None = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def save_cache(cache: dict, path: str | None = None) -> None:
    path = path or cache_path()
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + f".{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates(size: int, n_angles: int, resident_blocks: int):
    fs = [s for s in SPLITS if s == 1 or size // s >= 16]
    bs = [s for s in SPLITS if s == 1 or n_angles // s >= 8]
    grids = sorted({resident_blocks, max(1, resident_blocks // 2)}) + [-1]
    return [dict(fp_split=f, bp_split=b, grid_blocks=g) for f, b, g in itertools.product(fs, bs, grids)]


def choose(key: str, cands: list, measure, cache: dict | None = None, path: str | None = None) -> dict:
    """The cached choice for ``key``, else the candidate with the smallest
    ``measure(cand)`` (seconds), stored in the cache."""
    with _lock:
        cache = load_cache(path) if cache is None else cache
        if key in cache and isinstance(cache[key], dict) and "fp_split" in cache[key]:
            return cache[key]
        best, best_t = None, float("inf")
        for c in cands:
            t = measure(c)
            if t < best_t:
                best, best_t = dict(c), t
        best["ms"] = best_t * 1e3
        cache[key] = best
        save_cache(cache, path)
        return best


def tune_sirt(angles, rhozero: float, deltarho: float, numrhos: int, size: int, projections, nslices: int = 1,
              iterations: int = 6, path: str | None = None) -> dict:
    """Tuned launch shape for SIRT of this geometry (measured on the GPU)."""
    import torch

    from . import _lib
    from . import runtime as rt

    L = _lib.load()
    resident = int(L.synk_sirt_resident_blocks()) if hasattr(L, "synk_sirt_resident_blocks") else 0
    if resident <= 0:
        props = torch.cuda.get_device_properties(projections.device)
        resident = 2 * props.multi_processor_count
    key = bucket(size, angles.numel(), numrhos, nslices)

    def measure(c):
        args = (angles, rhozero, deltarho, numrhos, size, nslices, None, projections, iterations)
        kw = dict(fp_split=c["fp_split"], bp_split=c["bp_split"], grid_blocks=c["grid_blocks"])
        rt.sirt_slices(*args, **kw)                 # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rt.sirt_slices(*args, **kw)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3

    return choose(key, candidates(size, angles.numel(), resident), measure, path=path)
