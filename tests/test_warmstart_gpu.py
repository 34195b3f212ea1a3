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
    xs, ts = warmstart.make_dataset(prob, 384, seed=5, target_iters=300, chunk=128)
    net = UNet(256, 32, seed=0)
    hist = warmstart.train(net, xs, ts, epochs=6, batch=32, lr=1e-3)
    assert hist[-1] < hist[0]
    ev = warmstart.evaluate(net, prob, 32, seed=4242, budgets=(10, 20, 50), max_iters=200)
    assert ev["fallback_images"] == 0
    # the start is better than one plain update, and the gain is largest where
    # plain SIRT's own budget is short
    assert ev["warm_start_residual_mean"] < ev["plain_residual_after_1"]
    k10 = ev["rows"][0]
    assert k10["warm_iterations_mean"] < 0.7 * k10["plain_iterations_mean"], ev
