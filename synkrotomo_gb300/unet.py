"""U-Net warm starter on libsynk's tcgen05 kernels (``synk_unet_*`` of the C ABI).

The network maps the normalised backprojection C*A^T*R*b of a sinogram (one
SIRT update from zero) to a start image for SIRT.  Architecture: 4 levels,
32 base channels, 3x3 convolutions + ReLU, BF16 activations, FP32
accumulation, FP32 master weights, residual 1x1 head (see csrc/unet.cu).
"""
from __future__ import annotations

import ctypes

import torch

from . import runtime as rt

# (cin, cout) of the fourteen 3x3 convolutions, in parameter order
LAYERS = [(1, 32), (32, 32), (32, 64), (64, 64), (64, 128), (128, 128), (128, 256), (256, 256), (384, 128),
          (128, 128), (192, 64), (64, 64), (96, 32), (32, 32)]


def param_shapes():
    """[(name, shape)] of the flat FP32 parameter vector."""
    out = []
    for i, (ci, co) in enumerate(LAYERS):
        out.append((f"conv{i}.w", (co, 9 * ci)))
        out.append((f"conv{i}.b", (co,)))
    out.append(("head.w", (32,)))
    out.append(("head.b", (1,)))
    return out


class UNet:
    def __init__(self, size: int, max_batch: int, seed: int = 0, device: int | None = None):
        self.ctx = rt.context(device)
        self.size, self.max_batch = int(size), int(max_batch)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.synk_unet_new(self.ctx.handle, ctypes.byref(h), self.max_batch, self.size,
                                                  ctypes.c_uint64(seed)), "synk_unet_new")
        self._h = h
        self.nparams = int(self.ctx.lib.synk_unet_num_params(h))
        self.device = torch.device("cuda", self.ctx.device)
        self._loss = torch.zeros(1, dtype=torch.float64, device=self.device)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            try:
                self.ctx.lib.synk_unet_free(h)
            except Exception:
                pass
            self._h = None

    def params(self) -> torch.Tensor:
        out = torch.empty(self.nparams, dtype=torch.float32, device=self.device)
        ctx = rt.context(self.ctx.device)
        ctx.check(ctx.lib.synk_unet_params(ctx.handle, self._h, rt._ptr(out), 0), "synk_unet_params")
        return out

    def load(self, flat: torch.Tensor):
        flat = flat.to(self.device, torch.float32).contiguous()
        assert flat.numel() == self.nparams
        ctx = rt.context(self.ctx.device)
        ctx.check(ctx.lib.synk_unet_params(ctx.handle, self._h, rt._ptr(flat), 1), "synk_unet_params")

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        x = x.to(self.device, torch.float32).contiguous()
        b = x.numel() // (self.size * self.size)
        y = torch.empty_like(x)
        ctx = rt.context(self.ctx.device)
        for i in range(0, b, self.max_batch):
            nb = min(self.max_batch, b - i)
            n0 = i * self.size * self.size
            xs, ys = x.view(-1)[n0:], y.view(-1)[n0:]
            ctx.check(ctx.lib.synk_unet_forward(ctx.handle, self._h, rt._ptr(xs), rt._ptr(ys), nb), "synk_unet_forward")
        return y

    def train_step(self, x: torch.Tensor, target: torch.Tensor, lr: float = 1e-3, apply: bool = True) -> torch.Tensor:
        """One step; returns the batch loss as a device tensor (no host sync)."""
        x = x.to(self.device, torch.float32).contiguous()
        target = target.to(self.device, torch.float32).contiguous()
        b = x.numel() // (self.size * self.size)
        ctx = rt.context(self.ctx.device)
        ctx.check(ctx.lib.synk_unet_train_step(ctx.handle, self._h, rt._ptr(x), rt._ptr(target), b, float(lr),
                                               int(bool(apply)), rt._ptr(self._loss)), "synk_unet_train_step")
        return self._loss

    def gradients(self) -> torch.Tensor:
        out = torch.empty(self.nparams, dtype=torch.float32, device=self.device)
        ctx = rt.context(self.ctx.device)
        ctx.check(ctx.lib.synk_unet_gradients(ctx.handle, self._h, rt._ptr(out)), "synk_unet_gradients")
        return out
