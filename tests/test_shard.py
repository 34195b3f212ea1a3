"""Multi-rank split of independent SIRT work, on CPU with two gloo ranks.

The per-rank solver is the oracle (the GPU solver is the same call on each
rank's device); what is tested is the host logic: the partition, the gather
and the timing reduction. The sharded results must equal the single-process
oracle bit for bit, since every slice and problem is computed the same way
wherever it lands."""
import itertools
import math
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from oracle import cpu_ref
from synkrotomo_gb300 import phantom
from synkrotomo_gb300 import shard


def test_slice_ranges_cover_and_balance():
    for n, w in itertools.product([0, 1, 2, 7, 9, 64], [1, 2, 3, 8]):
        r = shard.slice_ranges(n, w)
        assert len(r) == w and r[0][0] == 0 and r[-1][1] == n
        assert all(r[k][1] == r[k + 1][0] for k in range(w - 1))
        sizes = [b - a for a, b in r]
        assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.slice_ranges(4, 0)


def _best_makespan(costs, world):
    best = math.inf
    for assign in itertools.product(range(world), repeat=len(costs)):
        loads = [0.0] * world
        for c, k in zip(costs, assign):
            loads[k] += c
        best = min(best, max(loads))
    return best


def test_lpt_bound_and_determinism():
    rng = np.random.default_rng(0)
    for trial in range(40):
        world = int(rng.integers(1, 4))
        costs = rng.integers(1, 50, size=int(rng.integers(0, 8))).astype(float).tolist()
        owner = shard.lpt_assign(costs, world)
        assert owner == shard.lpt_assign(costs, world)
        assert all(0 <= k < world for k in owner)
        loads = [0.0] * world
        for c, k in zip(costs, owner):
            loads[k] += c
        if costs:
            bound = (4.0 / 3.0 - 1.0 / (3.0 * world)) * _best_makespan(costs, world)
            assert max(loads) <= bound + 1e-9
    # a cost from the projector's work model: the big problem goes alone
    c = [shard.problem_cost(180, 363, 256), shard.problem_cost(30, 91, 64), shard.problem_cost(30, 91, 64)]
    assert shard.lpt_assign(c, 2) == [0, 1, 1]
    with pytest.raises(ValueError):
        shard.lpt_assign([1.0, -1.0], 2)


def test_gather_checks_ownership_single_rank():
    x = torch.arange(4, dtype=torch.float32)
    assert [t.tolist() for t in shard.gather_items({0: x, 1: x[:2]}, [0, 0])] == [x.tolist(), [0.0, 1.0]]
    with pytest.raises(ValueError):
        shard.gather_items({0: x}, [0, 0])
    with pytest.raises(TypeError):
        shard.gather_items({0: x.double()}, [0])
    assert shard.max_over_ranks(2.5) == 2.5


def _sirt3d_case(size=10, n_angles=8, iterations=4):
    g = phantom.geometry(size, n_angles)
    rhos = (np.float32(g.rhozero) + np.float32(g.deltarho) * np.arange(g.numrhos, dtype=np.float32)).astype(np.float32)
    stack = np.concatenate([cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos,
                                                      phantom.ellipse_phantom(size, seed=k)) for k in range(size)])
    return g.angles, rhos, stack.astype(np.float32), iterations, size


def _batch_case():
    probs = []
    for k, (n, a) in enumerate([(12, 10), (20, 16), (8, 5), (16, 12), (10, 7)]):
        g = phantom.geometry(n, a)
        img = phantom.ellipse_phantom(n, seed=100 + k)
        sino = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
        probs.append((g, np.zeros(n * n, np.float32), sino, 3 + k))
    return probs


def _cpu_slices(angles, rhos, part, iterations, size, nslices):
    return torch.from_numpy(cpu_ref.sirt3d(angles.numpy(), rhos.numpy(), part.numpy(), iterations, size,
                                           nslices=nslices))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    try:
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        cpu_ref.set_threads(1)
        # timing reduction: the slowest rank's time
        t = shard.max_over_ranks(1.5 + rank)
        # SIRT3D split by slices (10 slices over 2 ranks: 5 + 5)
        ang, rhos, stack, it, size = _sirt3d_case()
        vol = shard.sirt3d_sharded(torch.from_numpy(ang), torch.from_numpy(rhos), torch.from_numpy(stack), it,
                                   size, solve=_cpu_slices)
        # a ragged batch split by cost
        probs = _batch_case()
        costs = [shard.problem_cost(g.angles.size, g.numrhos, g.size, 1, it) for g, _, _, it in probs]

        def solve(idx):
            out = []
            for i in idx:
                g, x0, sino, iters = probs[i]
                out.append(torch.from_numpy(cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, x0, sino, iters)))
            return out

        res = shard.batch_sharded(costs, solve)
        q.put((rank, t, vol.numpy().copy(), [r.numpy().copy() for r in res], shard.lpt_assign(costs, world)))
        dist.barrier()
        dist.destroy_process_group()
    except Exception as e:   # report to the parent instead of hanging it
        q.put((rank, "error", repr(e), None, None))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_match_single_process():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    got = {}
    try:
        for _ in range(world):
            rank, t, vol, res, owner = q.get(timeout=240)
            assert t != "error", f"rank {rank}: {vol}"
            got[rank] = (t, vol, res, owner)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    ang, rhos, stack, it, size = _sirt3d_case()
    ref_vol = cpu_ref.sirt3d(ang, rhos, stack, it, size)
    probs = _batch_case()
    ref_res = [cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, x0, sino, iters) for g, x0, sino, iters in probs]
    for rank in range(world):
        t, vol, res, owner = got[rank]
        assert t == 2.5
        np.testing.assert_array_equal(vol, ref_vol)
        assert len(res) == len(ref_res)
        for a, b in zip(res, ref_res):
            np.testing.assert_array_equal(a, b)
        assert sorted(set(owner)) == [0, 1]          # both ranks got work
    assert got[0][3] == got[1][3]                    # same assignment on every rank


def _mismatch_worker(rank, world, port, q):
    import torch.distributed as dist
    try:
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        costs = [3.0, 1.0, 2.0] if rank == 0 else [3.0, 1.0, 2.0, 5.0]    # rank 1 sees another batch
        try:
            shard.batch_sharded(costs, lambda idx: [torch.zeros(2) for _ in idx])
            q.put((rank, "no error"))
        except ValueError as e:
            q.put((rank, "ValueError"))
        dist.destroy_process_group()
    except Exception as e:
        q.put((rank, repr(e)))


def test_ranks_with_different_assignments_fail_together():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_mismatch_worker, args=(k, world, port, q)) for k in range(world)]
    for p in procs:
        p.start()
    got = {}
    try:
        for _ in range(world):
            rank, what = q.get(timeout=240)
            got[rank] = what
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert got == {0: "ValueError", 1: "ValueError"}


def _local_fault_worker(rank, world, port, q, fault):
    import torch.distributed as dist
    try:
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        owner = [0, 1, 0, 1]
        local = {i: torch.zeros(3) for i in range(4) if owner[i] == rank}
        if rank == 1 and fault == "items":
            local[2] = torch.zeros(3)               # an item rank 0 owns
        if rank == 1 and fault == "dtype":
            local[1] = torch.zeros(3, dtype=torch.float64)
        try:
            shard.gather_items(local, owner)
            q.put((rank, "no error"))
        except (ValueError, TypeError) as e:
            q.put((rank, type(e).__name__))
        dist.destroy_process_group()
    except Exception as e:
        q.put((rank, repr(e)))


@pytest.mark.parametrize("fault,kind", [("items", "ValueError"), ("dtype", "TypeError")])
def test_a_local_fault_on_one_rank_fails_every_rank(fault, kind):
    """One rank passes a wrong item set or dtype: both ranks raise (none is
    left waiting in a collective)."""
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_local_fault_worker, args=(k, world, port, q, fault)) for k in range(world)]
    for p in procs:
        p.start()
    got = {}
    try:
        for _ in range(world):
            rank, what = q.get(timeout=240)
            got[rank] = what
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert got == {0: kind, 1: kind}


def test_sirt3d_sharded_non_cubic_stack_single_rank():
    """nslices != size: a stack of 3 slices of 10 x 10 through the driver
    equals the oracle's stack."""
    ang, rhos, _, it, size = _sirt3d_case()
    rng = np.random.default_rng(11)
    stack = rng.random(3 * ang.size * rhos.size).astype(np.float32)
    vol = shard.sirt3d_sharded(torch.from_numpy(ang), torch.from_numpy(rhos), torch.from_numpy(stack), it, size,
                               solve=_cpu_slices, nslices=3)
    ref = cpu_ref.sirt3d(ang, rhos, stack, it, size, nslices=3)
    np.testing.assert_array_equal(vol.numpy(), ref)
    with pytest.raises(ValueError):
        shard.sirt3d_sharded(torch.from_numpy(ang), torch.from_numpy(rhos), torch.from_numpy(stack), it, size,
                             solve=_cpu_slices, nslices=4)
