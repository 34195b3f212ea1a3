"""U-Net warm starter: tcgen05 forward/backward against the FP64 CPU oracle,
the fused Adam update against NumPy, and training on a fixed batch.

Tolerance: BF16 activations and gradients between layers give relative
errors of about 1e-2; a relative L2 error of 5e-2 per parameter tensor with a
cosine similarity above 0.999 overall separates that from any wrong index or
missing term (which gives O(1) errors)."""
import numpy as np
import pytest
import torch

from oracle import unet_ref
from synkrotomo_gb300 import phantom
from synkrotomo_gb300.unet import UNet, param_shapes

pytestmark = pytest.mark.gpu


def _inputs(B=2, N=256, seed=0):
    xs, ts = [], []
    for b in range(B):
        img = phantom.ellipse_phantom(N, seed + b)
        ts.append(img)
        rng = np.random.default_rng(seed + b)
        xs.append((0.6 * img + 0.05 * rng.standard_normal(img.size)).astype(np.float32))   # a blurry-noisy input
    return np.stack(xs).reshape(B, N, N), np.stack(ts).reshape(B, N, N)


def _rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_forward_matches_fp64_oracle(gpu):
    x, _ = _inputs()
    net = UNet(256, 2, seed=1)
    y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    params = unet_ref.unflatten(net.params().cpu())
    ref = unet_ref.forward(params, torch.from_numpy(x).double()).detach().numpy()
    # compare the learned correction (y - x), not the residual input itself
    assert _rel(y - x, ref - x) < 5e-2


def test_gradients_match_fp64_oracle(gpu):
    x, t = _inputs(seed=3)
    net = UNet(256, 2, seed=2)
    # a trained-looking network: push the head off its small init so every layer gets gradient
    p = net.params()
    p[-33:-1] = torch.linspace(-0.5, 0.5, 32, device="cuda")
    net.load(p)
    loss = net.train_step(torch.from_numpy(x), torch.from_numpy(t), apply=False)
    g = net.gradients().cpu().numpy().astype(np.float64)
    loss_ref, _, g_ref = unet_ref.loss_and_grads(net.params().cpu(), x, t)
    g_ref = g_ref.numpy()
    assert abs(float(loss.item()) - loss_ref) / loss_ref < 1e-2
    off = 0
    for name, shape in param_shapes():
        n = int(np.prod(shape))
        a, b = g[off:off + n], g_ref[off:off + n]
        if np.linalg.norm(b) > 1e-12:
            assert _rel(a, b) < 5e-2, name
        off += n
    cos = float(g @ g_ref / (np.linalg.norm(g) * np.linalg.norm(g_ref)))
    assert cos > 0.999


def test_fused_adam_matches_numpy(gpu):
    x, t = _inputs(seed=5)
    net = UNet(256, 2, seed=3)
    w0 = net.params().cpu().numpy().astype(np.float64)
    m = np.zeros_like(w0)
    v = np.zeros_like(w0)
    for step in (1, 2):
        net.train_step(torch.from_numpy(x), torch.from_numpy(t), apply=False)
        g = net.gradients().cpu().numpy().astype(np.float64)
        net.load(torch.from_numpy(w0.astype(np.float32)))   # same weights, so the next step sees the same g
        net_w = net.params()
        # the step with the Adam update, from the same weights
        net.train_step(torch.from_numpy(x), torch.from_numpy(t), lr=1e-3, apply=True)
        m = 0.9 * m + 0.1 * g
        v = 0.999 * v + 0.001 * g * g
        w_ref = w0 - 1e-3 * (m / (1 - 0.9 ** step)) / (np.sqrt(v / (1 - 0.999 ** step)) + 1e-8)
        w = net.params().cpu().numpy().astype(np.float64)
        assert np.max(np.abs(w - w_ref)) < 1e-5
        w0 = w
        del net_w


def test_training_reduces_the_loss(gpu):
    x, t = _inputs(B=4, seed=7)
    net = UNet(256, 4, seed=4)
    xs, ts = torch.from_numpy(x).cuda(), torch.from_numpy(t).cuda()
    first = float(net.train_step(xs, ts, lr=1e-3).item())
    for _ in range(30):
        last = float(net.train_step(xs, ts, lr=1e-3).item())
    assert last < 0.5 * first
