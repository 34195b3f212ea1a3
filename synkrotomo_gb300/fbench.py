"""Run the drop-in programs the way the reference runs its Futhark programs.

The reference times its programs with ``futhark bench --runs=10`` over the
datasets named in each program's header (Makefile:11-18,
``forwardprojection.fut:1-14``) and keeps the results as ``N;microseconds``
CSV files (``output/*/fut_fp.csv``, ``fut_bp.csv``).  Its compiled programs
read their arguments from standard input in Futhark's value format and print
the result.  This module offers both on top of the GPU drop-in classes:

* ``run_executable(name)``: ``python -m futhark.forwardprojection < data``
  reads ``main``'s arguments from standard input, runs it and prints the
  result as a Futhark value; ``-r N`` repeats the run, ``-t FILE`` writes each
  run's time in microseconds, ``-b`` prints binary.
* ``bench(name, datasets, runs)``: mean microseconds per dataset, as
  ``futhark bench`` reports them, and ``write_csv`` in the reference's
  ``N;us`` form (N = the digits that end the dataset's file name).
* ``generate(name, size, ...)``: a synthetic dataset for a program in its
  ``main`` argument layout, since the reference's datasets other than
  ``fpinputf32rad512`` are not shipped.

Timing follows Futhark's executables: the inputs are uploaded to the GPU
first, and a run is ``main`` plus a device synchronisation, timed with CUDA
events; the result stays on the device.

CLI: ``python -m synkrotomo_gb300.fbench bench forwardprojection data/* --csv fut_fp.csv``
and ``python -m synkrotomo_gb300.fbench generate forwardprojection 512 out``.
"""
from __future__ import annotations

import argparse
import math
import os
import re
import sys
from typing import Iterable, List, Sequence

import numpy as np

from . import fvalues

__all__ = ["PROGRAMS", "program", "parse_args_for", "run_executable", "bench", "write_csv", "generate"]

PROGRAMS = ("forwardprojection", "forwardprojection_sparse", "backprojection", "backprojection_sparse", "SIRT",
            "SIRT3D", "diff", "mse", "sanityCheck")


def program(name: str):
    """The drop-in class of a reference program, by the program's name."""
    if name not in PROGRAMS:
        raise KeyError(f"unknown program {name!r}; known: {', '.join(PROGRAMS)}")
    from . import dropin
    return getattr(dropin, name)


_SCALAR = {"f32": np.float32, "i32": np.int32, "bool": np.bool_}


def parse_args_for(name: str, values: Sequence) -> list:
    """Check ``values`` against ``main``'s declared parameter types and return
    them as numpy arrays / scalars (the executables reject a mismatch)."""
    params = program(name).entry_points["main"][0]
    if len(values) != len(params):
        raise fvalues.FormatError(f"{name}: main takes {len(params)} values, the input holds {len(values)}")
    out = []
    for i, (v, t) in enumerate(zip(values, params)):
        t = t.lstrip("*")
        a = np.asarray(v)
        if t.startswith("[]"):
            et = t[2:]
            if a.ndim != 1 or a.dtype != np.dtype(_SCALAR[et]):
                raise fvalues.FormatError(f"{name}: argument #{i} must be {t}, got {a.dtype}{list(a.shape)}")
            out.append(np.ascontiguousarray(a))
        else:
            if a.ndim != 0 or a.dtype != np.dtype(_SCALAR[t]):
                raise fvalues.FormatError(f"{name}: argument #{i} must be {t}, got {a.dtype}{list(a.shape)}")
            out.append(a[()])
    return out


def _upload(args: list, device: int) -> list:
    import torch
    dev = torch.device("cuda", device)
    return [torch.from_numpy(a).to(dev) if isinstance(a, np.ndarray) and a.ndim else a for a in args]


def _timed_runs(obj, args: list, runs: int) -> tuple:
    """Result of the last run and the microseconds of each run."""
    import torch
    times = []
    res = None
    for _ in range(max(1, runs)):
        st = torch.cuda.current_stream(obj.device)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(obj.device)
        e0.record(st)
        res = obj.main(*args)
        e1.record(st)
        torch.cuda.synchronize(obj.device)
        times.append(e0.elapsed_time(e1) * 1000.0)
    return res, times


def _result_value(res):
    if hasattr(res, "get"):
        return res.get()
    return res


def run_executable(name: str, argv: Sequence[str] | None = None) -> int:
    """Command-line behaviour of the compiled reference program ``name``."""
    ap = argparse.ArgumentParser(prog=f"python -m futhark.{name}",
                                 description=f"Run {name}.main on arguments read in Futhark's value format.")
    ap.add_argument("-r", "--runs", type=int, default=0, help="run main this many times (timed)")
    ap.add_argument("-t", "--write-runtime-to", metavar="FILE", help="write each run's microseconds to FILE")
    ap.add_argument("-b", "--binary-output", action="store_true", help="print the result in binary")
    ap.add_argument("-i", "--input", metavar="FILE", help="read the arguments from FILE instead of stdin")
    ap.add_argument("-d", "--device", type=int, default=0)
    a = ap.parse_args(argv)
    data = open(a.input, "rb").read() if a.input else sys.stdin.buffer.read()
    try:
        args = parse_args_for(name, fvalues.read_values(data))
    except fvalues.FormatError as e:
        print(f"Error: {e}", file=sys.stderr)
        return 1
    obj = program(name)(device=a.device)
    dev_args = _upload(args, a.device)
    if a.runs > 0:
        obj.main(*dev_args)   # warm-up: library load, allocator pools
    res, times = _timed_runs(obj, dev_args, a.runs)
    if a.write_runtime_to:
        with open(a.write_runtime_to, "w") as f:
            for t in times:
                f.write(f"{int(round(t))}\n")
    val = _result_value(res)
    if a.binary_output:
        sys.stdout.buffer.write(fvalues.write_binary([val]))
    else:
        sys.stdout.write(fvalues.write_text([val]))
    return 0


def dataset_size(path: str) -> int:
    """The N of a dataset file name (``fpinputf32rad512`` -> 512)."""
    m = re.search(r"(\d+)$", os.path.basename(path))
    if not m:
        raise ValueError(f"no trailing size in the dataset name {path!r}")
    return int(m.group(1))


def bench(name: str, datasets: Iterable[str], runs: int = 10, device: int = 0) -> List[tuple]:
    """[(N, mean_us, [us per run])] for each dataset, one warm-up run first."""
    obj = program(name)(device=device)
    rows = []
    for path in datasets:
        args = parse_args_for(name, fvalues.read_file(path))
        dev_args = _upload(args, device)
        obj.main(*dev_args)
        _, times = _timed_runs(obj, dev_args, runs)
        rows.append((dataset_size(path), float(np.mean(times)), times))
    return rows


def write_csv(rows: Iterable[tuple], path: str) -> None:
    """The reference's ``N;mean_us`` lines (output/*/fut_fp.csv)."""
    with open(path, "w") as f:
        for r in rows:
            f.write(f"{r[0]};{r[1]:.2f}\n")


def generate(name: str, size: int, out: str | None = None, n_angles: int | None = None,
             numrhos: int | None = None, iterations: int = 10, seed: int = 0, binary: bool = False,
             arc: float = math.pi) -> list:
    """A synthetic dataset for ``name``'s ``main``: a seeded random-ellipse
    phantom (forward, SIRT) or its sinogram (backward, SIRT, SIRT3D), angles
    uniform in [0, arc), numrhos = ceil(N*sqrt(2)), rhozero = -(numrhos-1)/2.
    Written to ``out`` (text, or binary) when given; returns the values."""
    from . import phantom
    if name.endswith("_sparse"):
        base = name[: -len("_sparse")]
        n_angles = n_angles or 30
    else:
        base = name
    n_angles = n_angles or size
    g = phantom.geometry(size, n_angles, numrhos, arc=arc)
    rz, dr = np.float32(g.rhozero), np.float32(g.deltarho)
    img = phantom.ellipse_phantom(size, seed)

    if base == "forwardprojection":
        vals = [g.angles, rz, dr, np.int32(g.numrhos), img]
    elif base in ("backprojection", "SIRT", "SIRT3D"):
        proj = _project(g, img)
        if base == "backprojection":
            vals = [g.angles, rz, dr, np.int32(size), proj]
        elif base == "SIRT":
            vals = [g.angles, rz, dr, np.zeros(size * size, np.float32), proj, np.int32(iterations)]
        else:
            rhos = (rz + dr * np.arange(g.numrhos, dtype=np.float32)).astype(np.float32)
            stack = np.concatenate([_project(g, phantom.ellipse_phantom(size, seed + k)) for k in range(size)])
            vals = [g.angles, rhos, stack, np.int32(iterations), np.int32(size)]
    elif base in ("diff", "mse", "sanityCheck"):
        rng = np.random.default_rng(seed)
        vals = [img, (img + rng.normal(0, 0.02, img.shape)).astype(np.float32)]
    else:
        raise KeyError(name)
    if out:
        with open(out, "wb" if binary else "w") as f:
            (fvalues.write_binary if binary else fvalues.write_text)(vals, f)
    return vals


def _project(g, img: np.ndarray) -> np.ndarray:
    """The sinogram of ``img`` by the GPU forward projector."""
    from . import dropin
    return dropin.forwardprojection().main(g.angles, np.float32(g.rhozero), np.float32(g.deltarho),
                                           np.int32(g.numrhos), img).get()


def _main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="futhark-bench-style timing and datasets for the drop-in programs")
    sub = ap.add_subparsers(dest="cmd", required=True)
    b = sub.add_parser("bench", help="mean microseconds of main per dataset")
    b.add_argument("program", choices=PROGRAMS)
    b.add_argument("datasets", nargs="+")
    b.add_argument("--runs", type=int, default=10)
    b.add_argument("--csv", help="write N;us lines here")
    g = sub.add_parser("generate", help="write a synthetic dataset in main's argument layout")
    g.add_argument("program", choices=PROGRAMS)
    g.add_argument("size", type=int)
    g.add_argument("out")
    g.add_argument("--angles", type=int)
    g.add_argument("--numrhos", type=int)
    g.add_argument("--iterations", type=int, default=10)
    g.add_argument("--seed", type=int, default=0)
    g.add_argument("--binary", action="store_true")
    a = ap.parse_args(argv)
    if a.cmd == "bench":
        rows = bench(a.program, a.datasets, a.runs)
        for n, us, _ in rows:
            print(f"{n};{us:.2f}")
        if a.csv:
            write_csv(rows, a.csv)
    else:
        generate(a.program, a.size, a.out, a.angles, a.numrhos, a.iterations, a.seed, a.binary)
    return 0


if __name__ == "__main__":
    sys.exit(_main())
