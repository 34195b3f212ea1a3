"""What the trained network gains over plain SIRT: after a short training on
GPU-generated pairs, SIRT started from the network's output reaches the
residual that plain zero-start SIRT reaches after its budget in far fewer
iterations, on held-out phantoms."""
import pytest
import torch

from synkrotomo_gb300 import warmstart
from synkrotomo_gb300.unet import UNet

pytestmark = pytest.mark.gpu


def test_ellipse_batch_matches_the_phantom_statistics(gpu):
    x = warmstart.ellipse_batch(64, 256, seed=3)
    assert x.shape == (64, 256 * 256)
    assert float(x.min()) >= 0.0 and 0.5 < float(x.max()) < 10.0
    y = warmstart.ellipse_batch(64, 256, seed=3)
    assert torch.equal(x, y)


def test_trained_warm_start_beats_plain_sirt(gpu):
    prob = warmstart.Problem(256, 60)
    xs, ts = warmstart.make_dataset(prob, 1024, seed=5, target_iters=300, chunk=256)
    net = UNet(256, 32, seed=0)
    hist = warmstart.train(net, xs, ts, epochs=8, batch=32, lr=1e-3)
    assert hist[-1] < hist[0]
    ev = warmstart.evaluate(net, prob, 32, seed=4242, budgets=(10, 20, 50), max_iters=200)
    assert ev["fallback_images"] == 0
    # the start is better than one plain update, and the gain is largest where
    # plain SIRT's own budget is short
    assert ev["warm_start_residual_mean"] < ev["plain_residual_after_1"]
    k10 = ev["rows"][0]
    assert k10["warm_iterations_mean"] < 0.7 * k10["plain_iterations_mean"], ev
    assert ev["rows"][1]["warm_iterations_mean"] < ev["rows"][1]["plain_iterations_mean"], ev


def test_warm_started_sirt_matches_the_oracles(gpu):
    """SIRT from a network's start image on the GPU against the oracles' SIRT
    from the same start: the FP32 C restatement (the reference's float32
    rounding) within 1e-5, and the FP64 restatement within 1e-4 on a geometry
    whose rays never run along pixel edges (half-integer rhozero: 364
    detectors)."""
    import numpy as np

    from oracle import cpu_ref, fut_ref

    prob = warmstart.Problem(256, 180)
    prob.g = warmstart.phantom.geometry(256, 180, numrhos=364)
    prob.angles = torch.from_numpy(prob.g.angles).cuda()
    xs, ts = warmstart.make_dataset(prob, 64, seed=9, target_iters=50, chunk=64)
    net = UNet(256, 32, seed=0)
    warmstart.train(net, xs, ts, epochs=2, batch=32, lr=1e-3)
    imgs = warmstart.ellipse_batch(1, 256, seed=31)
    b = prob.sinograms(imgs, seed=31)
    x1, _, _ = prob.sirt(b, 1)
    x0 = net.forward(x1.view(1, 256, 256)).view(1, -1)
    assert float((x0 - x1).abs().max()) > 0.0            # the network changed the start
    its = 30
    xg, _, _ = prob.sirt(b, its, start=x0)
    g = prob.g
    x0n, bn = x0.view(-1).cpu().numpy(), b.view(-1).cpu().numpy()
    x32 = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, x0n, bn, its).astype(np.float64)
    ops = fut_ref.SirtOperators(g.angles, g.rhozero, g.deltarho, g.numrhos, 256)
    x64 = ops.iterate(x0n, bn, its)
    xg = xg.view(-1).cpu().double().numpy()
    e32 = np.linalg.norm(xg - x32) / np.linalg.norm(x32)
    e64 = np.linalg.norm(xg - x64) / np.linalg.norm(x64)
    assert e32 < 1e-5, e32
    assert e64 < 1e-4, e64


def _prob_and_sinos(n=3, seed=61):
    prob = warmstart.Problem(256, 90, noise=0.0)
    b = prob.sinograms(warmstart.ellipse_batch(n, 256, seed=seed), seed=seed)
    return prob, b


def test_solve_falls_back_to_the_zero_start(gpu):
    """A network whose output is far off (head bias +1000) gives a start whose
    residual exceeds the zero start's: solve() must then run plain SIRT, bit
    for bit, and say so."""
    prob, b = _prob_and_sinos()
    net = UNet(256, 8, seed=1)
    p = net.params()
    p[-1] = 1000.0                                   # the head's bias
    net.load(p)
    g = prob.g
    r = warmstart.solve(net, prob.angles, g.rhozero, g.deltarho, b, tol=2e-2, max_iters=400, residuals=True)
    assert bool(r.fallback.all()) and float(r.start_residual.min()) > 1.0
    xp, _, dp = prob.sirt(b, 400, tol=2e-2)
    assert torch.equal(r.x, xp)
    assert torch.equal(r.iterations, dp)
    assert float((r.residuals[:, 0] - 1.0).abs().max()) < 1e-12   # the zero start's residual


def test_solve_is_the_warm_start_pipeline(gpu):
    """Without a fallback, solve() = SIRT from net(one SIRT update) to tol."""
    prob, b = _prob_and_sinos(seed=62)
    xs, ts = warmstart.make_dataset(prob, 64, seed=7, target_iters=50, chunk=64)
    net = UNet(256, 32, seed=0)
    warmstart.train(net, xs, ts, epochs=2, batch=32, lr=1e-3)
    g = prob.g
    r = warmstart.solve(net, prob.angles, g.rhozero, g.deltarho, b, tol=2e-2, max_iters=400)
    assert not bool(r.fallback.any())
    x1, _, _ = prob.sirt(b, 1)
    x0 = net.forward(x1.view(-1, 256, 256)).view(b.shape[0], -1)
    xw, _, dw = prob.sirt(b, 400, start=x0, tol=2e-2)
    assert torch.equal(r.x, xw) and torch.equal(r.iterations, dw)
    # a single flat sinogram is a batch of one
    r1 = warmstart.solve(net, prob.angles, g.rhozero, g.deltarho, b[1].cpu().numpy(), tol=2e-2, max_iters=400)
    assert r1.x.shape == (1, 256 * 256) and int(r1.iterations[0]) == int(dw[1])
    with pytest.raises(ValueError):
        warmstart.solve(net, prob.angles, g.rhozero, g.deltarho, b[:, :-1], tol=2e-2)


def test_checkpoint_round_trip_resumes_training(gpu, tmp_path):
    """save() with the Adam state, load_checkpoint() into a fresh network: the
    state is restored bit for bit and the next training step gives the same
    parameters (to the last bits: the weight gradients are summed with
    floating-point atomics, whose order varies).  The compact inference
    checkpoint gives the same forward output bit for bit."""
    prob, _ = _prob_and_sinos()
    xs, ts = warmstart.make_dataset(prob, 32, seed=8, target_iters=20, chunk=32)
    net = UNet(256, 16, seed=3)
    for _ in range(3):
        net.train_step(xs[:16].view(16, 256, 256), ts[:16].view(16, 256, 256), lr=1e-3)
    full = str(tmp_path / "full.npz")
    net.save(full, meta={"note": "test"})
    net2 = UNet(256, 16, seed=99)
    assert net2.load_checkpoint(full) == {"note": "test"}
    assert torch.equal(net2.params(), net.params())
    m1, v1, s1 = net.optimizer_state()
    m2, v2, s2 = net2.optimizer_state()
    assert s1 == s2 == 3 and torch.equal(m1, m2) and torch.equal(v1, v2)
    before = net.params()
    for n_ in (net, net2):
        n_.train_step(xs[16:].view(16, 256, 256), ts[16:].view(16, 256, 256), lr=1e-3)
    after, after2 = net.params(), net2.params()
    assert float((after - before).abs().max()) > 1e-5           # the step moved the weights
    assert float((after2 - after).abs().max()) < 1e-6
    small = str(tmp_path / "small.npz")
    net.save(small, compact=True)
    net3 = UNet(256, 16, seed=5)
    net3.load_checkpoint(small)
    x = xs[:4].view(4, 256, 256)
    assert torch.equal(net3.forward(x), net.forward(x))
