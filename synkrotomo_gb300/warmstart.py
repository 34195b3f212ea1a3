"""Learned warm start for SIRT: data, training and evaluation.

Pipeline (everything on the GPU, through libsynk):
  data      seeded random-ellipse phantoms -> forward projection -> Gaussian
            noise (sigma = 1 % of the sinogram maximum); input = one SIRT
            update from zero, i.e. the normalised backprojection C*A^T*R*b;
            target = SIRT after `target_iters` updates (1000)
  training  the U-Net (synkrotomo_gb300.unet) with MSE loss and Adam
  use       x0 = net(C*A^T*R*b); SIRT from x0 until the relative data
            residual ||Ax - b|| / ||b|| reaches r*, the residual plain
            zero-start SIRT reaches after `budget` iterations; when the warm
            start's own residual exceeds the zero start's (1.0), the zero
            start is used instead
The comparison (iterations and milliseconds to r*) is against plain
zero-start SIRT on the same sinograms.

Run ``python -m synkrotomo_gb300.warmstart --help`` for the full experiment.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np
import torch

from . import phantom
from . import runtime as rt
from .unet import UNet


def ellipse_batch(n: int, size: int, seed: int, n_ellipses: int = 10, device="cuda") -> torch.Tensor:
    """n random-ellipse phantoms [n, size*size] (float32, on the device):
    centres U[-0.6, 0.6]*N/2, semi-axes U[0.05, 0.4]*N/2, rotation U[0, pi),
    additive intensity U[0, 1]; seeded per batch."""
    g = torch.Generator(device="cpu").manual_seed(int(seed))
    p = torch.rand(n, n_ellipses, 6, generator=g, dtype=torch.float64).to(device)
    half = size / 2.0
    cx = (p[..., 0] * 1.2 - 0.6) * half
    cy = (p[..., 1] * 1.2 - 0.6) * half
    ax = (0.05 + 0.35 * p[..., 2]) * half
    ay = (0.05 + 0.35 * p[..., 3]) * half
    phi = p[..., 4] * math.pi
    val = p[..., 5]
    coords = torch.arange(size, device=device, dtype=torch.float64) - half + 0.5
    yy, xx = torch.meshgrid(coords, coords, indexing="ij")
    img = torch.zeros(n, size, size, device=device, dtype=torch.float64)
    for e in range(n_ellipses):
        c, s = torch.cos(phi[:, e])[:, None, None], torch.sin(phi[:, e])[:, None, None]
        dx, dy = xx[None] - cx[:, e, None, None], yy[None] - cy[:, e, None, None]
        u, v = dx * c + dy * s, -dx * s + dy * c
        inside = (u / ax[:, e, None, None]) ** 2 + (v / ay[:, e, None, None]) ** 2 <= 1.0
        img += inside * val[:, e, None, None]
    return img.float().reshape(n, size * size)


class Problem:
    """Geometry of one warm-start configuration."""

    def __init__(self, size: int, n_angles: int, noise: float = 0.01):
        self.size, self.n_angles, self.noise = int(size), int(n_angles), float(noise)
        self.g = phantom.geometry(self.size, self.n_angles)
        self.angles = torch.from_numpy(self.g.angles).cuda()

    def sinograms(self, imgs: torch.Tensor, seed: int) -> torch.Tensor:
        """[n, a*D] noisy sinograms of [n, N*N] images."""
        g = self.g
        out = torch.empty(imgs.shape[0], g.n_rays, device=imgs.device)
        for i in range(imgs.shape[0]):
            rt.forwardprojection(self.angles, g.rhozero, g.deltarho, g.numrhos, imgs[i], out=out[i])
        gen = torch.Generator(device=imgs.device).manual_seed(int(seed) + 99991)
        sigma = self.noise * out.amax(dim=1, keepdim=True)
        return out + sigma * torch.randn(out.shape, device=imgs.device, generator=gen)

    def sirt(self, sinos: torch.Tensor, iterations: int, start: torch.Tensor | None = None, tol: float = 0.0,
             residuals: bool = False):
        g = self.g
        n = sinos.shape[0]
        x, res, done = rt.sirt_slices(self.angles, g.rhozero, g.deltarho, g.numrhos, self.size, n,
                                      None if start is None else start.reshape(-1).contiguous(),
                                      sinos.reshape(-1).contiguous(), iterations, tol=tol, residuals=residuals)
        return x.view(n, -1), res, done


def make_dataset(prob: Problem, n: int, seed: int, target_iters: int = 1000, chunk: int = 256):
    """inputs (normalised backprojections) and targets (SIRT after target_iters)."""
    xs, ts = [], []
    for c0 in range(0, n, chunk):
        k = min(chunk, n - c0)
        imgs = ellipse_batch(k, prob.size, seed * 1000003 + c0)
        b = prob.sinograms(imgs, seed * 1000003 + c0)
        x1, _, _ = prob.sirt(b, 1)
        xt, _, _ = prob.sirt(b, target_iters)
        xs.append(x1)
        ts.append(xt)
    return torch.cat(xs), torch.cat(ts)


def lr_at(step: int, total: int, lr: float, warmup: int = 100, floor: float = 0.02) -> float:
    """Learning rate of a step: linear warm-up to lr over `warmup` steps, then
    cosine decay to floor*lr at the last step."""
    if step < warmup:
        return lr * (step + 1) / warmup
    t = (step - warmup) / max(1, total - warmup)
    return lr * (floor + (1.0 - floor) * 0.5 * (1.0 + math.cos(math.pi * min(1.0, t))))


def train(net: UNet, inputs: torch.Tensor, targets: torch.Tensor, epochs: int, batch: int = 32, lr: float = 1e-3,
          seed: int = 0, log=None, schedule: bool = True):
    """Adam on the MSE loss, mini-batches drawn without replacement each
    epoch; peak learning rate lr with warm-up and cosine decay (schedule=True)
    or constant.  Returns the mean loss of each epoch."""
    n = inputs.shape[0]
    N = net.size
    hist = []
    g = torch.Generator(device="cpu").manual_seed(seed)
    total = epochs * (n // batch)
    step = 0
    for ep in range(epochs):
        perm = torch.randperm(n, generator=g)
        losses = []
        for i in range(0, n - batch + 1, batch):
            idx = perm[i:i + batch].cuda()
            lr_s = lr_at(step, total, lr, warmup=max(1, min(100, total // 10))) if schedule else lr
            step += 1
            loss = net.train_step(inputs[idx].view(batch, N, N), targets[idx].view(batch, N, N), lr=lr_s)
            losses.append(loss.clone())
        ep_loss = float(torch.stack(losses).mean().item())
        hist.append(ep_loss)
        if log:
            log(f"epoch {ep}: loss {ep_loss:.6g}")
    return hist


class WarmResult:
    """Result of ``solve``: images x [n, N*N], updates applied [n], the
    residual of the network's start [n], which images fell back to the zero
    start [n], and optionally the residual histories [n, max_iters+1]."""

    def __init__(self, x, iterations, start_residual, fallback, residuals=None):
        self.x, self.iterations, self.start_residual = x, iterations, start_residual
        self.fallback, self.residuals = fallback, residuals


def solve(net: UNet, angles, rhozero: float, deltarho: float, sinograms, tol: float = 1e-3,
          max_iters: int = 8000, residuals: bool = False) -> WarmResult:
    """Warm-started SIRT of one or more sinograms of one geometry.

    ``sinograms``: one flat sinogram [a*numrhos] or a batch [n, a*numrhos]
    (float32; numpy or torch); numrhos = length / a, as SIRT.fut:18 derives
    it; the image side is the network's.  Steps, all on the GPU with no host
    round trip:
      1. x1 = one SIRT update from zero (C*A^T*R*b, the network's input);
      2. x0 = net(x1);
      3. the relative data residual ||A x0 - b|| / ||b|| of each start; where
         it exceeds the zero start's (1.0), that image starts from zero
         instead (the fallback);
      4. SIRT from x0 until the residual is at most ``tol`` or ``max_iters``
         updates (x <- x + C*A^T*R*(b - A*x), SIRT.fut:27-39; the start image
         plays the role of SIRT.fut:12's ``image``).
    """
    ang = rt.to_device_f32(angles, 0, "angles")
    b = sinograms if isinstance(sinograms, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(sinograms))
    if b.dtype != torch.float32:
        raise TypeError(f"sinograms must be float32 (got {b.dtype})")
    b = b.to(ang.device)
    if b.dim() == 1:
        b = b.view(1, -1)
    if b.dim() != 2:
        raise ValueError(f"sinograms must be [a*numrhos] or [n, a*numrhos] (got shape {tuple(b.shape)})")
    n, p = b.shape
    a = ang.numel()
    if a < 1 or p % a:
        raise ValueError(f"sinogram length {p} is not a multiple of {a} angles")
    numrhos = p // a
    N = net.size
    b = b.contiguous().view(-1)
    x1, _, _ = rt.sirt_slices(ang, rhozero, deltarho, numrhos, N, n, None, b, 1)
    x0 = net.forward(x1.view(n, N, N)).view(n, N * N)
    _, r0, _ = rt.sirt_slices(ang, rhozero, deltarho, numrhos, N, n, x0.view(-1), b, 0, residuals=True)
    start_res = r0[:, 0]
    fallback = ~(start_res <= 1.0)          # NaN falls back too
    x0 = torch.where(fallback[:, None], torch.zeros_like(x0), x0)
    x, res, done = rt.sirt_slices(ang, rhozero, deltarho, numrhos, N, n, x0.view(-1), b, int(max_iters),
                                  tol=float(tol), residuals=residuals)
    return WarmResult(x.view(n, N * N), done, start_res, fallback, res)


def headline(net: UNet, prob: "Problem", n: int = 64, seed: int = 777777, tol: float = 1e-3,
             max_iters: int = 8000, per_image: int = 16) -> dict:
    """Milliseconds and iterations to the relative residual ``tol``: plain
    zero-start SIRT against ``solve`` on n held-out seeded phantoms (the
    problem's geometry and noise), all n in one call each way, and the first
    ``per_image`` images solved one call each.  Every timed region is CUDA
    events on the current stream after one untimed run of the same call; the
    warm side includes the SIRT update that makes the network's input, the
    network and the fallback check."""
    g = prob.g
    imgs = ellipse_batch(n, prob.size, seed)
    b = prob.sinograms(imgs, seed)

    def plain(bs):
        return rt.sirt_slices(prob.angles, g.rhozero, g.deltarho, g.numrhos, prob.size, bs.shape[0], None,
                              bs.reshape(-1).contiguous(), max_iters, tol=tol)[2]

    def warm(bs):
        r = solve(net, prob.angles, g.rhozero, g.deltarho, bs, tol=tol, max_iters=max_iters)
        return r.iterations, r.fallback

    def timed(fn, bs):
        fn(bs)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        out = fn(bs)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1), out

    ms_plain, it_plain = timed(plain, b)
    ms_warm, (it_warm, fb) = timed(warm, b)
    pi_plain = pi_warm = 0.0
    ratios = []
    k = min(per_image, n)
    for i in range(k):
        tp, _ = timed(plain, b[i:i + 1])
        tw, _ = timed(warm, b[i:i + 1])
        pi_plain += tp
        pi_warm += tw
        ratios.append(tp / max(tw, 1e-9))
    it_plain = it_plain.float().cpu()
    it_warm = it_warm.float().cpu()
    return {"images": n, "size": prob.size, "angles": prob.n_angles, "noise": prob.noise, "target_residual": tol,
            "max_iterations": max_iters,
            "plain_iterations_mean": float(it_plain.mean()), "plain_iterations_median": float(it_plain.median()),
            "warm_iterations_mean": float(it_warm.mean()), "warm_iterations_median": float(it_warm.median()),
            "plain_not_reached": int((it_plain >= max_iters).sum()),
            "warm_not_reached": int((it_warm >= max_iters).sum()),
            "fallback_images": int(fb.sum().item()),
            "median_iteration_ratio": float(torch.median(it_plain / it_warm.clamp(min=1.0))),
            "batched_ms_plain": ms_plain, "batched_ms_warm": ms_warm, "speedup_batched": ms_plain / ms_warm,
            "per_image_images": k, "per_image_ms_plain": pi_plain, "per_image_ms_warm": pi_warm,
            "speedup_per_image": pi_plain / max(pi_warm, 1e-9),
            "speedup_per_image_median": float(torch.tensor(ratios).median()) if ratios else None}


def first_below(hist: torch.Tensor, target: torch.Tensor) -> torch.Tensor:
    """Per row, the first iteration k with hist[k] <= target (hist.shape[1] if none)."""
    ok = hist <= target[:, None]
    k = torch.where(ok.any(dim=1), ok.float().argmax(dim=1), torch.full_like(target, hist.shape[1]).long())
    return k


def evaluate(net: UNet, prob: Problem, n: int, seed: int, budgets=(10, 20, 50, 100, 200), max_iters: int = 600,
             abs_targets=(), per_image_count: int = 16):
    """Plain zero-start SIRT vs warm-started SIRT on n held-out images.

    For each plain budget K: r*_i = 1.01 x the residual plain SIRT reaches on
    image i after K iterations.  For each absolute target r (abs_targets, e.g.
    1e-3 on noise-free data): r*_i = r.  Iterations to r*_i come from full
    residual histories (plain and warm, one run each, max_iters iterations;
    an image that never reaches r*_i counts max_iters and is reported).
    Milliseconds are measured on batched runs that stop each image at its own
    r*_i when r* is absolute, and at the loosest r* of the batch otherwise; the
    warm run includes the normalised backprojection and the network.  Also,
    for the first per_image_count images solved one launch each to their own
    r*_i, the summed milliseconds (the cost a single-image caller sees)."""
    plain_len = max(max(budgets) if budgets else 0, max_iters if abs_targets else 0)
    imgs = ellipse_batch(n, prob.size, seed)
    b = prob.sinograms(imgs, seed)
    _, hp, _ = prob.sirt(b, plain_len, residuals=True)
    x1, _, _ = prob.sirt(b, 1)
    x0 = net.forward(x1.view(n, prob.size, prob.size)).view(n, -1)
    _, hw, _ = prob.sirt(b, max_iters, start=x0, residuals=True)
    fallback = hw[:, 0] > 1.0          # the warm start is worse than the zero start

    def timed(tol):
        ms = {}
        for label in ("plain", "warm"):
            for rep in range(2):                       # first run warms up
                torch.cuda.synchronize()
                t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                t0.record()
                start = None
                if label == "warm":
                    xa, _, _ = prob.sirt(b, 1)
                    start = net.forward(xa.view(n, prob.size, prob.size)).view(n, -1)
                _, _, done = prob.sirt(b, max_iters, start=start, tol=tol)
                t1.record()
                torch.cuda.synchronize()
            ms[label] = t0.elapsed_time(t1)
        return ms

    def per_image(rstar, count):
        """Summed ms of `count` images solved one launch each to their own r*
        (warm: one SIRT update, the network and the warm-started solve)."""
        ms = {"plain": 0.0, "warm": 0.0}
        for i in range(count):
            bi = b[i:i + 1]
            tol_i = float(rstar[i].item())
            for label in ("plain", "warm"):
                for rep in range(2):                   # first run warms up
                    torch.cuda.synchronize()
                    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    t0.record()
                    start = None
                    if label == "warm" and not bool(fallback[i]):
                        xa, _, _ = prob.sirt(bi, 1)
                        start = net.forward(xa.view(1, prob.size, prob.size)).view(1, -1)
                    prob.sirt(bi, max_iters, start=start, tol=tol_i)
                    t1.record()
                    torch.cuda.synchronize()
                ms[label] += t0.elapsed_time(t1)
        return ms

    def row(rstar, tol):
        it_plain = first_below(hp, rstar).float()
        it_warm = torch.where(fallback, it_plain, first_below(hw, rstar).float())
        ms = timed(tol)
        pim = per_image(rstar, min(per_image_count, n))
        return {"target_residual_mean": float(rstar.mean().item()),
                "plain_iterations_mean": float(it_plain.mean().item()),
                "warm_iterations_mean": float(it_warm.mean().item()),
                "plain_iterations_median": float(it_plain.median().item()),
                "warm_iterations_median": float(it_warm.median().item()),
                "plain_not_reached": int((it_plain >= hp.shape[1]).sum().item()),
                "warm_not_reached": int((it_warm >= hw.shape[1]).sum().item()),
                "speedup_iterations": float(it_plain.mean().item() / max(it_warm.mean().item(), 1e-9)),
                "batched_ms_plain": ms["plain"], "batched_ms_warm": ms["warm"],
                "speedup_ms": ms["plain"] / max(ms["warm"], 1e-9),
                "per_image_images": min(per_image_count, n),
                "per_image_ms_plain": pim["plain"], "per_image_ms_warm": pim["warm"],
                "speedup_per_image_ms": pim["plain"] / max(pim["warm"], 1e-9)}

    rows = []
    for Kb in budgets:
        rstar = hp[:, Kb] * 1.01
        rows.append({"budget": Kb, **row(rstar, float(rstar.max().item()))})
    for r in abs_targets:
        rows.append({"residual": float(r), **row(torch.full_like(hp[:, 0], float(r)), float(r))})
    return {"n": n, "size": prob.size, "angles": prob.n_angles, "noise": prob.noise,
            "warm_start_residual_mean": float(hw[:, 0].mean().item()),
            "plain_residual_after_1": float(hp[:, 1].mean().item()),
            "fallback_images": int(fallback.sum().item()), "rows": rows}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--eval", type=int, default=512)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--batch", type=int, default=32)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--angles", type=int, default=180)
    ap.add_argument("--target-iters", type=int, default=1000)
    ap.add_argument("--noise", type=float, default=0.01, help="Gaussian noise, fraction of each sinogram's max")
    ap.add_argument("--budgets", default="10,20,50,100,200", help="plain budgets K (r* = 1.01 r_plain(K))")
    ap.add_argument("--abs-targets", default="", help="absolute residual targets, e.g. 1e-3 (noise-free data)")
    ap.add_argument("--max-iters", type=int, default=600)
    ap.add_argument("--constant-lr", action="store_true", help="no warm-up / cosine decay")
    ap.add_argument("--mix-angles", type=int, default=0,
                    help="also train on this angle count (half the phantoms each) for the sparse-view case")
    ap.add_argument("--skip-sparse", action="store_true", help="no sparse-view evaluation")
    ap.add_argument("--sparse-size", type=int, default=512)
    ap.add_argument("--sparse-angles", type=int, default=90)
    ap.add_argument("--out", default="")
    ap.add_argument("--save", default="", help="write the trained network as an inference checkpoint (.npz)")
    ap.add_argument("--save-full", default="", help="write weights and Adam state (.npz, resumable)")
    ap.add_argument("--skip-eval", action="store_true")
    args = ap.parse_args(argv)
    torch.cuda.set_device(0)
    log = lambda m: print(m, flush=True)   # noqa: E731
    budgets = tuple(int(v) for v in args.budgets.split(",") if v)
    abs_t = tuple(float(v) for v in args.abs_targets.split(",") if v)
    prob = Problem(args.size, args.angles, noise=args.noise)
    t0 = time.time()
    if args.mix_angles:
        # half the pairs at the evaluation geometry, half at the extra angle count
        # (same image size, so one network sees both streak patterns)
        half = args.train // 2
        xa, ta = make_dataset(prob, half, seed=1, target_iters=args.target_iters)
        pmix = Problem(args.size, args.mix_angles, noise=args.noise)
        xb, tb = make_dataset(pmix, args.train - half, seed=2, target_iters=args.target_iters)
        xs, ts = torch.cat([xa, xb]), torch.cat([ta, tb])
        del xa, ta, xb, tb
    else:
        xs, ts = make_dataset(prob, args.train, seed=1, target_iters=args.target_iters)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    log(f"dataset {args.train} x {args.size}^2 in {t_data:.1f} s")
    net = UNet(args.size, args.batch, seed=0)
    t0 = time.time()
    hist = train(net, xs, ts, args.epochs, args.batch, args.lr, log=log, schedule=not args.constant_lr)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    del xs, ts
    meta = {"phantoms": args.train, "noise": args.noise, "target_iters": args.target_iters, "size": args.size,
            "angles": args.angles, "mix_angles": args.mix_angles, "epochs": args.epochs, "batch": args.batch,
            "lr": args.lr, "final_loss": hist[-1] if hist else None, "data_seed": 1, "init_seed": 0,
            "train_s": t_train, "data_s": t_data}
    if args.save:
        net.save(args.save, meta=meta, compact=True)
    if args.save_full:
        net.save(args.save_full, meta=meta, optimizer=True)
    res = {"train": {"phantoms": args.train, "noise": args.noise, "target_iters": args.target_iters,
                     "angles": args.angles, "mix_angles": args.mix_angles, "epochs": args.epochs, "batch": args.batch,
                     "lr": args.lr,
                     "loss_per_epoch": hist, "data_s": t_data, "train_s": t_train,
                     "steps": args.epochs * (args.train // args.batch)}}
    if args.skip_eval:
        if args.out:
            with open(args.out, "w") as f:
                json.dump(res, f, indent=1)
        return res
    res["eval_dense"] = evaluate(net, prob, args.eval, seed=777777, budgets=budgets, max_iters=args.max_iters,
                                 abs_targets=abs_t)
    log(json.dumps(res["eval_dense"]))
    if not args.skip_sparse:
        sparse = Problem(args.sparse_size, args.sparse_angles, noise=args.noise)
        net512 = UNet(args.sparse_size, 8, seed=0)
        net512.load(net.params())
        res["eval_sparse_view"] = evaluate(net512, sparse, args.eval, seed=888888, budgets=budgets,
                                           max_iters=args.max_iters, abs_targets=abs_t)
        log(json.dumps(res["eval_sparse_view"]))
    if args.out:
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)
    return res


if __name__ == "__main__":
    main()
