"""Uneven batches of independent SIRT problems in one persistent launch, and
the autotuner of the launch shape."""
import math

import numpy as np
import pytest
import torch

from oracle import cpu_ref
from synkrotomo_gb300 import autotune, phantom
from synkrotomo_gb300 import runtime as rt
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def _make(size, a, seed, arc=math.pi, nslices=1, noise=0.01):
    g = phantom.geometry(size, a, arc=arc)
    sinos = []
    for s in range(nslices):
        img = phantom.ellipse_phantom(size, seed + 100 * s)
        b = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)
        sinos.append(phantom.add_noise(b, seed + s, noise))
    return g, np.concatenate(sinos)


def test_uneven_batch_matches_single_problem_runs(gpu):
    # sizes, angle counts (some limited-angle), slice counts and iteration counts all differ
    specs = [(64, 60, math.pi, 1, 20), (32, 90, 2 * math.pi / 3, 1, 35), (48, 17, math.pi, 2, 10),
             (96, 45, math.pi, 1, 25), (16, 8, 2 * math.pi / 3, 3, 40), (80, 120, math.pi, 1, 5)]
    problems, refs = [], []
    for i, (size, a, arc, ns, its) in enumerate(specs):
        g, b = _make(size, a, seed=i, arc=arc, nslices=ns)
        problems.append(rt.Problem(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, size, _dev(b), its,
                                   nslices=ns, residuals=True))
        per = b.reshape(ns, -1)
        refs.append([cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(size * size, np.float32), per[s], its)
                     for s in range(ns)])
    rt.sirt_batch(problems)
    for p, ref, spec in zip(problems, refs, specs):
        x = p.out.cpu().numpy().reshape(p.nslices, -1)
        for s in range(p.nslices):
            assert rel_l2(x[s], ref[s]) < 1e-5, spec
        assert np.all(p.done.cpu().numpy() == spec[4])
        r = p.residuals.cpu().numpy()
        assert np.all(np.isfinite(r)) and np.all(np.diff(r, axis=1) <= 1e-6)


def test_batch_stopping_rule_per_problem(gpu):
    specs = [(64, 60, 0), (32, 30, 1), (48, 40, 2)]
    probs, tols = [], []
    for size, a, seed in specs:
        g, b = _make(size, a, seed, noise=0.0)
        p = rt.Problem(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, size, _dev(b), 60, residuals=True)
        probs.append(p)
    rt.sirt_batch(probs)
    hist = [p.residuals.cpu().numpy()[0] for p in probs]
    tol = max(h[25] for h in hist) * 1.0001
    probs2 = []
    for (size, a, seed) in specs:
        g, b = _make(size, a, seed, noise=0.0)
        probs2.append(rt.Problem(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, size, _dev(b), 60))
    rt.sirt_batch(probs2, tol=tol)
    for p, h in zip(probs2, hist):
        k = int(p.done.item())
        assert k == next(i for i, v in enumerate(h) if v <= tol)


def test_autotuner_picks_a_valid_shape_and_caches_it(gpu, tmp_path):
    g, b = _make(64, 48, 0)
    path = str(tmp_path / "tune.json")
    ang, bd = _dev(g.angles), _dev(b)
    c = autotune.tune_sirt(ang, g.rhozero, g.deltarho, g.numrhos, 64, bd, path=path)
    # grid_blocks: a persistent grid, or -1 for the phase-split engine
    assert c["fp_split"] in (1, 2, 4, 8) and c["bp_split"] in (1, 2, 4, 8)
    assert c["grid_blocks"] >= 1 or c["grid_blocks"] == -1
    assert autotune.load_cache(path)[autotune.bucket(64, 48, g.numrhos, 1)] == c
    x, _, _ = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 64, 1, None, bd, 20,
                             fp_split=c["fp_split"], bp_split=c["bp_split"], grid_blocks=c["grid_blocks"])
    ref = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, np.zeros(64 * 64, np.float32), b, 20)
    assert rel_l2(x.cpu().numpy(), ref) < 1e-5


def test_sirt_plan_graph_replay(gpu):
    # two problems captured once in a CUDA graph; replays after refilling the
    # sinograms in place give the same images as direct batched solves on the
    # same engine (a captured plan runs the persistent kernel on the resident
    # grid, which picks its tile shapes for that grid)
    specs = [(64, 40, 0), (32, 24, 1)]
    probs, sinos = [], []
    for size, a, seed in specs:
        g, b = _make(size, a, seed)
        p = rt.Problem(_dev(g.angles), g.rhozero, g.deltarho, g.numrhos, size, _dev(b), 25, residuals=True)
        probs.append(p)
        sinos.append((g, b))
    plan = rt.SirtPlan(probs)
    for rep in range(2):
        for p, (g, b) in zip(probs, sinos):
            p.projections.copy_(_dev(b * (1.0 + 0.5 * rep)))
        plan.launch()
        outs = [p.out.clone() for p in probs]
        direct = [rt.Problem(p.angles, p.rhozero, p.deltarho, p.numrhos, p.size, p.projections.clone(), 25)
                  for p in probs]
        rt.sirt_batch(direct, grid_blocks=rt.resident_blocks())
        for o, d in zip(outs, direct):
            assert torch.equal(o, d.out)
        default = [rt.Problem(p.angles, p.rhozero, p.deltarho, p.numrhos, p.size, p.projections.clone(), 25)
                   for p in probs]
        rt.sirt_batch(default)
        for o, d in zip(outs, default):
            assert rel_l2(o.cpu().numpy(), d.out.cpu().numpy()) < 1e-6
        for p in probs:
            assert int(p.done[0].item()) == 25


def test_sharded_drivers_single_rank_gpu(gpu):
    """Without a process group the multi-rank drivers run the whole job on this
    GPU: SIRT3D through the sharded driver equals SIRT3D bit for bit, and a
    cost-split batch equals one batched launch."""
    from synkrotomo_gb300 import shard
    size, a, its = 32, 24, 12
    g, b = _make(size, a, seed=7, nslices=size)
    rhos = (np.float32(g.rhozero) + np.float32(g.deltarho) * np.arange(g.numrhos, dtype=np.float32))
    ang_d, rhos_d, b_d = _dev(g.angles), _dev(rhos.astype(np.float32)), _dev(b)
    ref = rt.sirt3d(ang_d, rhos_d, b_d, its, size)
    vol = shard.sirt3d_sharded(ang_d, rhos_d, b_d, its, size)
    assert torch.equal(vol, ref)

    specs = [(64, 60, 15), (32, 30, 9), (48, 40, 11)]
    made = [_make(s, n, seed=20 + i) for i, (s, n, _) in enumerate(specs)]
    costs = [shard.problem_cost(n, g.numrhos, s, 1, it) for (s, n, it), (g, _) in zip(specs, made)]

    def solve(idx):
        probs = [rt.Problem(_dev(made[i][0].angles), made[i][0].rhozero, made[i][0].deltarho, made[i][0].numrhos,
                            specs[i][0], _dev(made[i][1]), specs[i][2]) for i in idx]
        return [p.out for p in rt.sirt_batch(probs)]

    res = shard.batch_sharded(costs, solve)
    ref = solve(list(range(len(specs))))
    for x, y in zip(res, ref):
        assert torch.equal(x, y)
