"""FP64 CPU restatement of the U-Net warm starter (csrc/unet.cu).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``): the checker of the
tcgen05 forward and backward kernels.  The network has no counterpart in the
reference; this module states its definition independently, on PyTorch's CPU
float64 operators with autograd for the gradients.
"""
from __future__ import annotations

import torch
import torch.nn.functional as F

LAYERS = [(1, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128), (128, 256), (256, 256), (384, 128),
          (128, 128), (192, 64), (64, 64), (96, 32), (32, 32)]


def unflatten(flat):
    """Parameter tensors (float64, requires_grad) from the flat vector."""
    flat = torch.as_tensor(flat, dtype=torch.float64).flatten()
    out, off = [], 0
    for ci, co in LAYERS:
        w = flat[off:off + 9 * ci * co].view(co, 3, 3, ci).permute(0, 3, 1, 2).clone()   # [co][ci][3][3]
        off += 9 * ci * co
        b = flat[off:off + co].clone()
        off += co
        out += [w, b]
    out += [flat[off:off + 32].clone(), flat[off + 32:off + 33].clone()]
    assert off + 33 == flat.numel()
    for t in out:
        t.requires_grad_(True)
    return out


def flatten_grads(params):
    g = []
    for i, (ci, co) in enumerate(LAYERS):
        g.append(params[2 * i].grad.permute(0, 2, 3, 1).reshape(-1))     # back to [co][tap][ci]
        g.append(params[2 * i + 1].grad.reshape(-1))
    g += [params[-2].grad.reshape(-1), params[-1].grad.reshape(-1)]
    return torch.cat(g)


def forward(params, x):
    """x [B][N][N] float64 -> y [B][N][N]."""
    c = lambda t, i: F.relu(F.conv2d(t, params[2 * i], params[2 * i + 1], padding=1))   # noqa: E731
    x0 = x[:, None]
    e1 = c(c(x0, 0), 1)
    e2 = c(c(F.max_pool2d(e1, 2), 2), 3)
    e3 = c(c(F.max_pool2d(e2, 2), 4), 5)
    e4 = c(c(F.max_pool2d(e3, 2), 6), 7)
    up = lambda t: F.interpolate(t, scale_factor=2, mode="nearest")   # noqa: E731
    d3 = c(c(torch.cat([up(e4), e3], 1), 8), 9)
    d2 = c(c(torch.cat([up(d3), e2], 1), 10), 11)
    d1 = c(c(torch.cat([up(d2), e1], 1), 12), 13)
    y = x0 + torch.einsum("bchw,c->bhw", d1, params[-2])[:, None] + params[-1]
    return y[:, 0]


def loss_and_grads(flat, x, target):
    params = unflatten(flat)
    y = forward(params, torch.as_tensor(x, dtype=torch.float64))
    loss = ((y - torch.as_tensor(target, dtype=torch.float64)) ** 2).mean()
    loss.backward()
    return float(loss.detach()), y.detach(), flatten_grads(params)
