"""Independent SIRT work split across ranks (one process per GPU).

The slices of a SIRT3D volume (futhark/SIRT3D.fut:18-29 maps SIRT over them)
and the problems of a batch share nothing while they iterate, so a multi-GPU
run partitions them and exchanges data only once, when the results are
gathered at the end. No collective runs on the data path.

* ``slice_ranges``: contiguous, balanced slice ranges (equal cost per slice).
* ``lpt_assign``: problems of unequal cost to ranks by longest-processing-time
  first (each problem, largest first, to the least-loaded rank); the cost of a
  problem is ``problem_cost`` = slices x iterations x (a*D*N + a*N*N), the
  row-steps of the forward projector plus the pixel-angle pairs of the
  backprojector.
* ``gather_items``: every rank gets every rank's results (one all-gather of
  padded flat buffers, after a check that all ranks hold the same assignment
  and one all-reduce of the lengths).
* ``sirt3d_sharded`` / ``batch_sharded``: the two drivers.
* ``max_over_ranks``: the timing reduction of a weak-scaling run.

Without an initialised process group every function acts as a single rank.
The assignment is a pure function of the inputs, so every rank computes the
same one without talking to the others.
"""
from __future__ import annotations

import heapq
import zlib
from typing import Callable, Dict, List, Sequence, Tuple

import numpy as np
import torch

__all__ = ["world_rank", "slice_ranges", "problem_cost", "lpt_assign", "max_over_ranks", "gather_items",
           "sirt3d_sharded", "batch_sharded"]


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def world_rank(group=None) -> Tuple[int, int]:
    """(world size, rank); (1, 0) without a process group."""
    d = _dist()
    if d is None:
        return 1, 0
    return d.get_world_size(group), d.get_rank(group)


def _comm_device(group=None) -> torch.device:
    d = _dist()
    if d is not None and d.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def slice_ranges(nslices: int, world: int) -> List[Tuple[int, int]]:
    """[start, stop) per rank; the first ``nslices % world`` ranks take one more."""
    if world < 1:
        raise ValueError(f"world size must be positive (got {world})")
    if nslices < 0:
        raise ValueError(f"slice count must be non-negative (got {nslices})")
    base, extra = divmod(int(nslices), int(world))
    out, s = [], 0
    for k in range(world):
        n = base + (1 if k < extra else 0)
        out.append((s, s + n))
        s += n
    return out


def problem_cost(n_angles: int, numrhos: int, size: int, nslices: int = 1, iterations: int = 1) -> float:
    """Work of one SIRT problem: per slice and iteration the forward projector
    walks a*D rays over N rows and the backprojector visits a*N*N
    (pixel, angle) pairs."""
    a, d, n = int(n_angles), int(numrhos), int(size)
    return float(nslices) * float(max(iterations, 1)) * (a * d * n + a * n * n)


def lpt_assign(costs: Sequence[float], world: int) -> List[int]:
    """Rank of each item: items in decreasing cost (ties by index) each go to
    the rank with the least assigned cost (ties to the lower rank). The
    makespan is at most (4/3 - 1/(3*world)) of the best partition."""
    if world < 1:
        raise ValueError(f"world size must be positive (got {world})")
    c = [float(x) for x in costs]
    if any(not np.isfinite(x) or x < 0 for x in c):
        raise ValueError("costs must be finite and non-negative")
    order = sorted(range(len(c)), key=lambda i: (-c[i], i))
    heap = [(0.0, k) for k in range(world)]
    owner = [0] * len(c)
    for i in order:
        load, k = heapq.heappop(heap)
        owner[i] = k
        heapq.heappush(heap, (load + c[i], k))
    return owner


def max_over_ranks(value: float, group=None) -> float:
    """The largest ``value`` over the ranks (the slowest rank's time)."""
    d = _dist()
    if d is None:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=_comm_device(group))
    d.all_reduce(t, op=d.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_items(local: Dict[int, torch.Tensor], owner: Sequence[int], group=None,
                 dtype: torch.dtype = torch.float32) -> List[torch.Tensor]:
    """Every item's flat result on every rank, in item order.

    ``local`` maps the indices this rank owns (``owner[i] == rank``) to its
    results; lengths may differ per item. The buffers travel on the process
    group's device (CUDA for NCCL, host for gloo) and the results are views of
    the gathered buffers."""
    world, rank = world_rank(group)
    n = len(owner)
    mine = {i for i in range(n) if owner[i] == rank}
    wrong_items = set(local) != mine
    wrong_dtype = [i for i, t in local.items() if t.dtype != dtype]

    def raise_local():
        if wrong_items:
            raise ValueError(f"rank {rank} holds items {sorted(local)} but owns {sorted(mine)}")
        if wrong_dtype:
            i = wrong_dtype[0]
            raise TypeError(f"item {i} is {local[i].dtype}, expected {dtype}")

    if world == 1:
        raise_local()
        return [local[i].reshape(-1) for i in range(n)]
    d = _dist()
    dev = _comm_device(group)
    # Every rank must hold the same assignment (it is computed, not exchanged)
    # and its own items in the right dtype.  One MAX reduction carries a
    # checksum of the assignment (as +sig and -sig) and the ranks' local
    # failures, so that all ranks raise together instead of one rank raising
    # while the others wait in the next collective.
    sig = float(zlib.crc32(np.asarray(owner, dtype=np.int64).tobytes())) + 2.0 ** 32 * n
    chk = torch.tensor([sig, -sig, float(wrong_items), float(bool(wrong_dtype))], dtype=torch.float64, device=dev)
    d.all_reduce(chk, op=d.ReduceOp.MAX, group=group)
    if wrong_items or wrong_dtype:
        raise_local()
    if chk[2].item() or chk[3].item():
        kind = ValueError if chk[2].item() else TypeError
        raise kind("another rank holds a wrong item set or dtype for the gather")
    if chk[0].item() != -chk[1].item():
        raise ValueError("the ranks hold different item assignments (different costs or item counts)")
    lens = torch.zeros(max(n, 1), dtype=torch.int64, device=dev)
    for i, t in local.items():
        lens[i] = t.numel()
    d.all_reduce(lens, group=group)
    lens = [int(v) for v in lens.cpu().tolist()][:n]
    totals = [0] * world
    for i in range(n):
        totals[owner[i]] += lens[i]
    buf = torch.zeros(max(max(totals), 1), dtype=dtype, device=dev)
    off = 0
    for i in sorted(mine):
        buf[off:off + lens[i]] = local[i].reshape(-1).to(dev)
        off += lens[i]
    bufs = [torch.empty_like(buf) for _ in range(world)]
    d.all_gather(bufs, buf, group=group)
    out: List[torch.Tensor] = [None] * n   # type: ignore[list-item]
    offs = [0] * world
    for i in range(n):
        k = owner[i]
        out[i] = bufs[k][offs[k]:offs[k] + lens[i]]
        offs[k] += lens[i]
    return out


def _gpu_slices(angles, rhos, projections, iterations, size, nslices):
    """SIRT of ``nslices`` slices on this rank's GPU, with SIRT3D's geometry
    (rhozero = rhos[0], deltarho = rhos[1] - rhos[0] in float32)."""
    from . import runtime as rt
    rh = rhos[:2].detach().cpu().numpy().astype(np.float32)
    rhozero = float(rh[0])
    deltarho = float(np.float32(rh[1]) - np.float32(rh[0]))
    out, _, _ = rt.sirt_slices(angles, rhozero, deltarho, rhos.numel(), size, nslices, None, projections,
                               iterations)
    return out


def sirt3d_sharded(angles, rhos, projections, iterations: int, size: int, solve: Callable | None = None,
                   group=None, nslices: int | None = None) -> torch.Tensor:
    """SIRT3D (``size`` slices of ``size``x``size``, or ``nslices`` slices
    for a non-cubic stack) with the slices split over the ranks; every rank
    returns the whole volume.

    ``solve(angles, rhos, projections_part, iterations, size, nslices)``
    reconstructs a contiguous run of slices (default: this rank's GPU)."""
    world, rank = world_rank(group)
    solve = solve or _gpu_slices
    a, r = int(angles.numel()), int(rhos.numel())
    ns = int(size) if nslices is None else int(nslices)
    if ns < 1:
        raise ValueError(f"nslices must be positive (got {ns})")
    if r < 2:
        raise ValueError(f"rhos needs at least two detector positions (got {r})")
    per = a * r
    if projections.numel() != ns * per:
        raise ValueError(f"projections has {projections.numel()} values, expected slices*a*r = {ns * per}")
    ranges = slice_ranges(ns, world)
    owner = [k for k, (s0, s1) in enumerate(ranges) for _ in range(s0, s1)]
    s0, s1 = ranges[rank]
    n2 = int(size) * int(size)
    local = {}
    if s1 > s0:
        part = solve(angles, rhos, projections[s0 * per:s1 * per], int(iterations), int(size), s1 - s0)
        part = part.reshape(-1)
        for j in range(s0, s1):
            local[j] = part[(j - s0) * n2:(j - s0 + 1) * n2]
    return torch.cat(gather_items(local, owner, group, dtype=torch.float32))


def batch_sharded(costs: Sequence[float], solve: Callable[[List[int]], List[torch.Tensor]],
                  group=None) -> List[torch.Tensor]:
    """A batch of independent problems split by ``lpt_assign``.

    ``solve(indices)`` solves this rank's problems (typically in one
    ``runtime.sirt_batch`` launch) and returns their flat float32 results in
    the order given; every rank returns every problem's result."""
    world, rank = world_rank(group)
    owner = lpt_assign(costs, world)
    mine = [i for i in range(len(owner)) if owner[i] == rank]
    res = solve(mine) if mine else []
    if len(res) != len(mine):
        raise ValueError(f"solve returned {len(res)} results for {len(mine)} problems")
    return gather_items(dict(zip(mine, res)), owner, group, dtype=torch.float32)
