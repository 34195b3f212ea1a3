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
