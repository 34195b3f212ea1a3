"""U-Net warm starter on libsynk's tcgen05 kernels (``synk_unet_*`` of the C ABI).

The network maps the normalised backprojection C*A^T*R*b of a sinogram (one
SIRT update from zero) to a start image for SIRT.  Architecture: 4 levels,
32 base channels, 3x3 convolutions + ReLU, BF16 activations, FP32
accumulation, FP32 master weights, residual 1x1 head (see csrc/unet.cu).
"""
from __future__ import annotations

import ctypes
import json

import numpy as np
import torch

from . import runtime as rt

CHECKPOINT_FORMAT = "synkrotomo-gb300 unet checkpoint 1"

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


def _bf16_mask() -> np.ndarray:
    """Parameters the forward pass uses in BF16: the weights of convolutions
    1..13 (the tensor-core layers); the Cin = 1 input layer, the biases and
    the head stay FP32."""
    mask = []
    for i, (ci, co) in enumerate(LAYERS):
        mask.append(np.full(co * 9 * ci, i > 0))
        mask.append(np.zeros(co, bool))
    mask.append(np.zeros(33, bool))
    return np.concatenate(mask)


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

    def optimizer_state(self):
        """(m, v, step): Adam's first and second moments (device, FP32, the
        parameter layout) and the number of Adam steps taken."""
        m = torch.empty(self.nparams, dtype=torch.float32, device=self.device)
        v = torch.empty_like(m)
        step = ctypes.c_int64(0)
        ctx = rt.context(self.ctx.device)
        ctx.check(ctx.lib.synk_unet_optimizer_state(ctx.handle, self._h, rt._ptr(m), rt._ptr(v), ctypes.byref(step),
                                                    0), "synk_unet_optimizer_state")
        return m, v, int(step.value)

    def load_optimizer_state(self, m: torch.Tensor, v: torch.Tensor, step: int):
        m = m.to(self.device, torch.float32).contiguous()
        v = v.to(self.device, torch.float32).contiguous()
        if m.numel() != self.nparams or v.numel() != self.nparams:
            raise ValueError(f"optimizer state has {m.numel()}/{v.numel()} values, expected {self.nparams}")
        st = ctypes.c_int64(int(step))
        ctx = rt.context(self.ctx.device)
        ctx.check(ctx.lib.synk_unet_optimizer_state(ctx.handle, self._h, rt._ptr(m), rt._ptr(v), ctypes.byref(st),
                                                    1), "synk_unet_optimizer_state")

    def save(self, path: str, optimizer: bool = True, meta: dict | None = None, compact: bool = False):
        """Write a checkpoint (.npz).

        ``optimizer``: also Adam's moments and step count, so that training
        resumes where it stopped.  ``compact``: an inference checkpoint: the
        weights of the thirteen tensor-core convolutions in BF16 (the
        precision the forward pass uses them in, rounded the same way, so the
        network's outputs are unchanged), everything else in FP32, no
        optimizer state."""
        flat = self.params().cpu().numpy()
        out = {"format": np.array(CHECKPOINT_FORMAT), "layers": np.array(LAYERS, dtype=np.int32),
               "size": np.int32(self.size), "meta": np.array(json.dumps(meta or {}))}
        if compact:
            mask = _bf16_mask()
            bits = flat.view(np.uint32).astype(np.uint64)
            # round to nearest even, as the engine's FP32 -> BF16 conversion does
            rounded = ((bits + 0x7FFF + ((bits >> 16) & 1)) >> 16).astype(np.uint16)
            out["bf16_weights"] = rounded[mask]
            out["fp32_rest"] = flat[~mask]
        else:
            out["params"] = flat
            if optimizer:
                m, v, step = self.optimizer_state()
                out["adam_m"] = m.cpu().numpy()
                out["adam_v"] = v.cpu().numpy()
                out["adam_step"] = np.int64(step)
        np.savez_compressed(path, **out)

    def load_checkpoint(self, path: str) -> dict:
        """Load a checkpoint written by ``save`` (the weights, and Adam's state
        when it holds one); returns its metadata."""
        z = np.load(path)
        if str(z["format"]) != CHECKPOINT_FORMAT:
            raise ValueError(f"{path}: not a {CHECKPOINT_FORMAT!r} file")
        if not np.array_equal(z["layers"], np.array(LAYERS, dtype=np.int32)):
            raise ValueError(f"{path}: layer shapes differ from this network's")
        if "params" in z:
            flat = z["params"].astype(np.float32)
        else:
            mask = _bf16_mask()
            flat = np.empty(mask.size, np.float32)
            flat[mask] = (z["bf16_weights"].astype(np.uint32) << 16).view(np.float32)
            flat[~mask] = z["fp32_rest"]
        if flat.size != self.nparams:
            raise ValueError(f"{path}: {flat.size} parameters, expected {self.nparams}")
        self.load(torch.from_numpy(flat))
        if "adam_m" in z:
            self.load_optimizer_state(torch.from_numpy(z["adam_m"]), torch.from_numpy(z["adam_v"]),
                                      int(z["adam_step"]))
        return json.loads(str(z["meta"]))

    def gradients(self) -> torch.Tensor:
        out = torch.empty(self.nparams, dtype=torch.float32, device=self.device)
        ctx = rt.context(self.ctx.device)
        ctx.check(ctx.lib.synk_unet_gradients(ctx.handle, self._h, rt._ptr(out)), "synk_unet_gradients")
        return out
