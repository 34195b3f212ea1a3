"""Benchmark of the projection path on one GB300 (or N replicas under torchrun).

Workload: the dense projector pair of the projector microbench -- N=2048
image, 2048 angles in [0, pi), 2897 detectors, deltarho 1 -- on a seeded
random-ellipse phantom (forward projection) and a U[0,1) sinogram
(backprojection).  One step = one A*x (forward projection) plus one A^T*y
(backprojection) through the library's C ABI.

value: FP/BP GB/s = compulsory bytes of the step (image and sinogram read and
written, 8*(N^2 + a*D)) / device time, inputs resident in HBM, L2 flushed
before every step.  e2e: the same metric through the public drop-in API
(futhark.forwardprojection / futhark.backprojection) from pinned host arrays,
host<->device copies inside the timed region.

--impl reference times the reference's CPU path (the FP32 C restatement of
the Futhark programs, oracle/cpu_ref.c in its host-tuned build, every host
core) on the same workload: whole steps, every angle, nothing extrapolated.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

N_SIZE, N_ANGLES, N_DET = 2048, 2048, 2897     # the projector microbench's dense configuration
METRIC = "SIRT ms to rel. residual 1e-3: warm-start vs plain, 1 GB300; FP/BP GB/s"
LEGS = ("proj", "e2e", "sirt", "csr", "unet", "warm", "shard", "cpu")   # default legs; "batch", "stack", "sparse" on request
WARM_CHECKPOINT = os.path.join(ROOT, "synkrotomo_gb300", "checkpoints", "unet_n256_a180_noisefree.npz")


def set_workload(size, angles, detectors):
    """Smaller cases of the same workload (profiling); the defaults are the benchmark."""
    global N_SIZE, N_ANGLES, N_DET
    N_SIZE, N_ANGLES = int(size), int(angles)
    N_DET = int(detectors) if detectors else int(math.ceil(N_SIZE * math.sqrt(2.0)))


def workload_name():
    return (f"projector microbench, dense on-the-fly: N={N_SIZE} image, {N_ANGLES} angles in [0,pi), "
            f"{N_DET} detectors, deltarho=1")


def bench_config(n_gpus):
    """The workload description both arms print (same dict for the GPU arm and
    the reference arm)."""
    return {"workload": workload_name(), "image": N_SIZE, "angles": N_ANGLES, "detectors": N_DET,
            "step": "forward projection + backprojection",
            "l2": "flushed (512 MB write) before every step on the GPU; inputs (40.5 MB) exceed no cache on the host",
            "parallelism": f"replicas x{n_gpus}"}


def step_bytes():
    return 8 * (N_SIZE * N_SIZE + N_ANGLES * N_DET)


def flops_fp():
    # 14 flops per ray-row step (forwardprojection.fut:32-56; FMA=2, add/mul/div=1)
    return 14.0 * N_ANGLES * N_DET * N_SIZE


def flops_bp(rpp=2):
    # 13 flops per (pixel, line) + 13 per ray evaluation (backprojection.fut:49-64)
    return (13.0 + 13.0 * rpp) * N_SIZE * N_SIZE * N_ANGLES


def workload(seed=0):
    from synkrotomo_gb300 import phantom
    g = phantom.geometry(N_SIZE, N_ANGLES, numrhos=N_DET)
    img = phantom.ellipse_phantom(N_SIZE, seed)
    sino = np.random.default_rng(seed + 1).random(N_ANGLES * N_DET).astype(np.float32)
    return g, img, sino


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


# ---------------------------------------------------------------------------
# CPU leg (oracle/cpu_ref.c: test infrastructure, used here only as the timed
# stand-in for the reference's CPU build)
# ---------------------------------------------------------------------------

def cpu_reference_step(seed=0):
    """One whole step of the workload (forward projection of the image and
    backprojection of the sinogram over all angles) by the CPU port on every
    host core, timed build: seconds for FP, BP and the step."""
    from oracle import cpu_ref
    cpu_ref.use_build("timed")
    cores = host_cores()
    cpu_ref.set_threads(cores)
    g, img, sino = _cpu_workload(seed)
    t0 = time.perf_counter()
    cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, N_DET, img)
    t1 = time.perf_counter()
    cpu_ref.backprojection(g.angles, g.rhozero, g.deltarho, N_SIZE, sino)
    t2 = time.perf_counter()
    return {"fp_s": t1 - t0, "bp_s": t2 - t1, "step_s": t2 - t0, "cores": cores}


_CPU_WL = {}


def _cpu_workload(seed):
    if seed not in _CPU_WL:
        _CPU_WL[seed] = workload(seed)
    return _CPU_WL[seed]


def cpu_flags():
    """The timed CPU build's compiler flags (oracle/Makefile)."""
    try:
        r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "flags"], capture_output=True,
                           text=True, timeout=30)
        for line in r.stdout.splitlines():
            if line.strip().startswith("timed:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return "unknown"


def cpu_sirt_cfg0(iterations=200):
    """Plain SIRT on the N=128 configuration (128 angles, 182 detectors, 1 %
    noise, 200 iterations) by the CPU port on all host cores: seconds for the
    full run (the reference's own CPU-runnable case, timed whole)."""
    from oracle import cpu_ref

    from synkrotomo_gb300 import phantom
    cpu_ref.use_build("timed")
    cores = host_cores()
    cpu_ref.set_threads(cores)
    g = phantom.geometry(128, 128)
    img = phantom.ellipse_phantom(128, 0)
    b = phantom.add_noise(cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img), 0, 0.01)
    x0 = np.zeros(128 * 128, np.float32)
    t0 = time.perf_counter()
    cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, x0, b, iterations)
    return {"s": time.perf_counter() - t0, "iterations": iterations, "cores": cores}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu_index = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            # nvidia-smi takes a moment to start: wait for its first sample so
            # that the samples taken inside the timed region are its own
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None
        self.start = len(self.lines)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # the samples taken during the region (else the last one before its end)
        inside = self.lines[self.start:] or self.lines[-1:]
        for line in inside:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": smax, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def run_gpu(args, rank, world):
    import torch

    from synkrotomo_gb300 import runtime as rt
    from synkrotomo_gb300 import shard

    dev = torch.device("cuda", torch.cuda.current_device())
    g, img, sino = workload(seed=rank)
    ang_d = torch.from_numpy(g.angles).to(dev)
    img_d = torch.from_numpy(img).to(dev)
    sino_d = torch.from_numpy(sino).to(dev)
    fp_out = torch.empty(N_ANGLES * N_DET, device=dev)
    bp_out = torch.empty(N_SIZE * N_SIZE, device=dev)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)   # 512 MB > 129 MB L2
    stream = torch.cuda.current_stream(dev)

    def step():
        rt.forwardprojection(ang_d, g.rhozero, g.deltarho, N_DET, img_d, out=fp_out)
        rt.backprojection(ang_d, g.rhozero, g.deltarho, N_SIZE, sino_d, out=bp_out)

    for _ in range(args.warmup):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(dev.index) as clk:
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))         # L2 flush outside the timed events
            e0, e1, e2 = ev[i]
            e0.record(stream)
            rt.forwardprojection(ang_d, g.rhozero, g.deltarho, N_DET, img_d, out=fp_out)
            e1.record(stream)
            rt.backprojection(ang_d, g.rhozero, g.deltarho, N_SIZE, sino_d, out=bp_out)
            e2.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    rt.context(dev.index).sync()
    fp_ms = [a.elapsed_time(b) for a, b, _ in ev]
    bp_ms = [b.elapsed_time(c) for _, b, c in ev]
    step_ms = sum(fp_ms) / len(fp_ms) + sum(bp_ms) / len(bp_ms)
    if world > 1:
        step_ms = shard.max_over_ranks(step_ms)
        torch.distributed.barrier()

    # end to end through the public API, pinned host buffers
    e2e = run_e2e(args, g, img, sino, dev) if "e2e" in args.legs else None
    sirt = run_sirt_cfg0(dev) if (rank == 0 and "sirt" in args.legs) else None
    csr = run_csr_cfg1(dev) if (rank == 0 and "csr" in args.legs) else None
    batch = run_batch_cfg3(dev) if (rank == 0 and "batch" in args.legs) else None
    stack = run_stack_cfg2(dev) if (rank == 0 and "stack" in args.legs) else None
    sparse = run_sparseview(dev) if (rank == 0 and "sparse" in args.legs) else None
    unet = run_unet(dev) if (rank == 0 and "unet" in args.legs) else None
    warm = run_warm(dev) if (rank == 0 and "warm" in args.legs) else None
    shardleg = run_sirt3d_sharded(dev, world) if "shard" in args.legs else None
    return {"sparse": sparse, "unet": unet, "warm": warm, "shard": shardleg, "step_ms": step_ms, "fp_ms": statistics.median(fp_ms), "bp_ms": statistics.median(bp_ms),
            "wall_s": wall, "clocks": clk.summary(), "e2e": e2e, "sirt": sirt, "csr": csr, "batch": batch,
            "stack": stack,
            "sms": torch.cuda.get_device_properties(dev).multi_processor_count}


def run_e2e(args, g, img, sino, dev):
    import torch

    from futhark import backprojection, forwardprojection

    def pinned(a):
        t = torch.empty(a.size, dtype=torch.float32, pin_memory=True)
        t.numpy()[:] = a
        return t.numpy()

    ang_h, img_h, sino_h = pinned(g.angles), pinned(img), pinned(sino)
    fpm, bpm = forwardprojection.forwardprojection(), backprojection.backprojection()

    def step():
        s = fpm.main(ang_h, g.rhozero, g.deltarho, N_DET, img_h).get()
        b = bpm.main(ang_h, g.rhozero, g.deltarho, N_SIZE, sino_h).get()
        return s, b

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    h2d = 4 * (2 * N_ANGLES + N_SIZE * N_SIZE + N_ANGLES * N_DET)
    d2h = 4 * (N_ANGLES * N_DET + N_SIZE * N_SIZE)
    return {"ms": ms, "h2d": h2d, "d2h": d2h}


def run_sirt_cfg0(dev):
    """Plain SIRT on the reference's CPU-runnable configuration (N=128, 128
    angles, 182 detectors, 1 % noise): ms for 200 iterations, and ms to the
    relative residual that 200 plain iterations reach."""
    import torch

    from synkrotomo_gb300 import phantom
    from synkrotomo_gb300 import runtime as rt

    g = phantom.geometry(128, 128)
    img = torch.from_numpy(phantom.ellipse_phantom(128, 0)).to(dev)
    ang = torch.from_numpy(g.angles).to(dev)
    b = rt.forwardprojection(ang, g.rhozero, g.deltarho, g.numrhos, img).cpu().numpy()
    b = torch.from_numpy(phantom.add_noise(b, 0, 0.01)).to(dev)
    x0 = torch.zeros(128 * 128, device=dev)
    _, res, _ = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 128, 1, x0, b, 200, residuals=True)
    target = float(res[0, 200].item()) * 1.01
    out = {}
    for label, tol in (("200_iterations", 0.0), ("to_residual", target)):
        for _ in range(3):
            rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 128, 1, x0, b, 200, tol=tol)
        torch.cuda.synchronize()
        ts = []
        for _ in range(10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _, _, done = rt.sirt_slices(ang, g.rhozero, g.deltarho, g.numrhos, 128, 1, x0, b, 200, tol=tol)
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        out[label] = {"ms": statistics.median(ts), "iterations": int(done.item())}
    out["target_residual"] = target
    return out


def _ellipsoid_stack_gpu(size, n_slices, seed, dev, n_ellipsoids=12):
    """phantom.ellipsoid_volume's stack (the same seeded ellipsoids and rule),
    evaluated on the GPU in float64: [n_slices, size*size] float32."""
    import math

    import torch

    rng = np.random.default_rng(seed)
    half, zh = size / 2.0, n_slices / 2.0
    coords = torch.arange(size, dtype=torch.float64, device=dev) - half + 0.5
    y, x = torch.meshgrid(coords, coords, indexing="ij")
    params = []
    for _ in range(n_ellipsoids):
        cx, cy = rng.uniform(-0.6, 0.6, 2) * half
        cz = rng.uniform(-0.6, 0.6) * zh
        ax, ay = rng.uniform(0.05, 0.4, 2) * half
        az = rng.uniform(0.05, 0.4) * zh
        phi = rng.uniform(0.0, math.pi)
        val = rng.uniform(0.0, 1.0)
        params.append((cx, cy, cz, ax, ay, az, math.cos(phi), math.sin(phi), val))
    vol = torch.zeros(n_slices, size, size, dtype=torch.float32, device=dev)
    for z in range(n_slices):
        zc = z - zh + 0.5
        sl = torch.zeros(size, size, dtype=torch.float64, device=dev)
        for cx, cy, cz, ax, ay, az, c, s_, val in params:
            dz = ((zc - cz) / az) ** 2
            if dz > 1.0:
                continue
            u = (x - cx) * c + (y - cy) * s_
            v = -(x - cx) * s_ + (y - cy) * c
            sl += (((u / ax) ** 2 + (v / ay) ** 2) <= 1.0 - dz).to(torch.float64) * val
        vol[z] = sl.to(torch.float32)
    return vol.reshape(n_slices, size * size)


def run_sirt3d_sharded(dev, world, slices=512, iterations=10, seed=0):
    """The slice stack of the SIRT3D configuration (512 slices of 512 x 512,
    360 angles, 725 detectors, 1 % noise) split over the ranks by
    shard.sirt3d_sharded (contiguous slice ranges, one SIRT launch per rank,
    one all-gather of the results at the end): all slices, `iterations`
    updates each (strong scaling: the stack is fixed).  Returns the slowest
    rank's milliseconds and the whole job's slice-iterations per second."""
    import torch

    from synkrotomo_gb300 import phantom, shard
    from synkrotomo_gb300 import runtime as rt

    N, a, D = 512, 360, 725
    ns = int(slices)
    g = phantom.geometry(N, a, numrhos=D)
    ang = torch.from_numpy(g.angles).to(dev)
    rhos = torch.from_numpy((np.float32(g.rhozero) + np.arange(D, dtype=np.float32)).astype(np.float32)).to(dev)
    vol = _ellipsoid_stack_gpu(N, ns, seed, dev)
    proj = torch.empty(ns * a * D, dtype=torch.float32, device=dev)
    for z in range(ns):     # every rank makes the same stack (same seeds)
        b = proj[z * a * D:(z + 1) * a * D]
        rt.forwardprojection(ang, g.rhozero, g.deltarho, D, vol[z], out=b)
        gen = torch.Generator(device=dev).manual_seed(seed * 1000 + z)
        b += torch.randn(b.shape, device=dev, generator=gen) * (0.01 * float(b.max()))
    del vol
    shard.sirt3d_sharded(ang, rhos, proj, 1, N, nslices=ns)          # warm-up
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    volr = shard.sirt3d_sharded(ang, rhos, proj, iterations, N, nslices=ns)
    e1.record()
    torch.cuda.synchronize()
    ms = shard.max_over_ranks(e0.elapsed_time(e1))
    assert volr.numel() == ns * N * N
    return {"slices": ns, "slices_per_rank": -(-ns // world), "iterations": iterations, "ranks": world,
            "ms": ms, "us_per_slice_iteration": 1e3 * ms * world / (ns * iterations),
            "slice_iterations_per_s": ns * iterations / (ms * 1e-3), "scaling": "strong",
            "split": "contiguous slice ranges, one all-gather of the results"}


def run_csr_cfg1(dev, reps=20):
    """CSR SpMV on the sparse projector configuration (N=512, 512 angles, 725
    detectors): GB/s of the compulsory traffic 8*nnz + 4*(rows+1) + 4*cols +
    4*rows per A*x (column vector gathered once) and the same for A^T*y."""
    import torch

    from synkrotomo_gb300 import phantom
    from synkrotomo_gb300 import runtime as rt

    g = phantom.geometry(512, 512, numrhos=725)
    t0 = time.perf_counter()
    m = rt.SystemMatrix(torch.from_numpy(g.angles).to(dev), g.rhozero, g.deltarho, g.numrhos, 512)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    x = torch.from_numpy(phantom.ellipse_phantom(512, 0)).to(dev)
    y = torch.rand(m.rows, device=dev)
    ax = torch.empty(m.rows, device=dev)
    aty = torch.empty(m.cols, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, device=dev)
    out = {"nnz": m.nnz, "rows": m.rows, "cols": m.cols, "build_s": build_s}
    for name, fn, rows, cols in (("Ax", lambda: m.matvec(x, ax), m.rows, m.cols),
                                 ("ATy", lambda: m.rmatvec(y, aty), m.cols, m.rows)):
        for _ in range(3):
            fn()
        ts = []
        for _ in range(reps):
            flush.fill_(0.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        ms = statistics.median(ts)
        nbytes = 8 * m.nnz + 8 * (rows + 1) + 4 * cols + 4 * rows   # int64 row pointers
        out[name] = {"ms": ms, "GB/s": nbytes / (ms * 1e-3) / 1e9, "bytes": nbytes}
    del m
    return out


def run_batch_cfg3(dev, seed=0, n_problems=64, iterations=150):
    """The uneven batch: 64 independent problems, N from {128,...,1024}, angle
    counts from {60,...,1024}, a quarter limited-angle ([0, 2pi/3)),
    ceil(N*sqrt(2)) detectors, 0.5-2 % noise, 150 iterations, in one launch;
    compared with the same problems run one launch each."""
    import torch

    from synkrotomo_gb300 import phantom
    from synkrotomo_gb300 import runtime as rt

    rng = np.random.default_rng(seed)
    probs_spec = []
    for i in range(n_problems):
        N = int(rng.choice([128, 256, 384, 512, 768, 1024]))
        a = int(rng.choice([60, 90, 180, 360, 720, 1024]))
        limited = rng.random() < 0.25
        noise = float(rng.uniform(0.005, 0.02))
        probs_spec.append((N, a, limited, noise))
    problems = []
    work = 0.0
    for i, (N, a, limited, noise) in enumerate(probs_spec):
        g = phantom.geometry(N, a, arc=(2 * math.pi / 3) if limited else math.pi)
        ang = torch.from_numpy(g.angles).to(dev)
        img = torch.from_numpy(phantom.ellipse_phantom(N, seed + i)).to(dev)
        b = rt.forwardprojection(ang, g.rhozero, g.deltarho, g.numrhos, img)
        b = b + torch.randn_like(b) * (noise * float(b.max()))
        problems.append(rt.Problem(ang, g.rhozero, g.deltarho, g.numrhos, N, b, iterations))
        work += (N * N * a + a * g.numrhos * N) * iterations
    torch.cuda.synchronize()
    rt.sirt_batch(problems)            # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    rt.sirt_batch(problems)
    e1.record()
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1)
    e0.record()
    for p in problems:
        rt.sirt_batch([p])
    e1.record()
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1)
    return {"problems": n_problems, "iterations": iterations, "ms_one_launch": batch_ms,
            "ms_one_launch_per_problem": seq_ms, "pixel_angle_and_ray_row_steps": work,
            "sizes": sorted({s[0] for s in probs_spec}), "angle_counts": sorted({s[1] for s in probs_spec})}


def run_stack_cfg2(dev, nslices=64, iterations=100, seed=0):
    """The slice stack (512 x 512 slices, 360 angles in [0,pi), 725 detectors,
    1 % noise, 100 iterations) for `nslices` of the 512 slices in one
    persistent launch; ms for the full 512-slice stack scaled linearly."""
    import torch

    from synkrotomo_gb300 import phantom
    from synkrotomo_gb300 import runtime as rt

    N = 512
    g = phantom.geometry(N, 360, numrhos=725)
    ang = torch.from_numpy(g.angles).to(dev)
    vol = phantom.ellipsoid_volume(N, 512, seed)[256 - nslices // 2: 256 + nslices // 2]
    sinos = []
    for z in range(nslices):
        b = rt.forwardprojection(ang, g.rhozero, g.deltarho, g.numrhos, torch.from_numpy(vol[z]).to(dev))
        sinos.append(b + torch.randn_like(b) * (0.01 * float(b.max())))
    b = torch.cat(sinos)
    prob = rt.Problem(ang, g.rhozero, g.deltarho, g.numrhos, N, b, iterations, nslices=nslices)
    rt.sirt_batch([prob])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    rt.sirt_batch([prob])
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    return {"slices_run": nslices, "iterations": iterations, "ms": ms, "ms_512_slices_scaled": ms * 512 / nslices,
            "ms_per_slice_iteration": ms / (nslices * iterations)}


def run_sparseview(dev, size=512, detectors=725, counts=(1, 5, 10, 20, 30, 45, 60, 95), reps=20):
    """The sparse-view programs (forward/backprojection_sparse, datasets of 1 to
    95 angles in [0, pi)) at N=512, 725 detectors: median microseconds per call
    and the rate per ray-row step / per (pixel, angle), inputs resident."""
    import torch

    from synkrotomo_gb300 import phantom
    from synkrotomo_gb300 import runtime as rt

    img = torch.from_numpy(phantom.ellipse_phantom(size, 0)).to(dev)
    out = {}
    for a in counts:
        g = phantom.geometry(size, a, numrhos=detectors)
        ang = torch.from_numpy(g.angles).to(dev)
        sino = torch.rand(a * detectors, device=dev)
        fo = torch.empty(a * detectors, device=dev)
        bo = torch.empty(size * size, device=dev)
        res = {}
        for name, fn in (("fp", lambda: rt.forwardprojection(ang, g.rhozero, g.deltarho, detectors, img, out=fo,
                                                             sparse=True)),
                         ("bp", lambda: rt.backprojection(ang, g.rhozero, g.deltarho, size, sino, out=bo,
                                                          sparse=True))):
            for _ in range(3):
                fn()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                fn()
                e1.record()
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1) * 1e3)
            res[name + "_us"] = statistics.median(ts)
        res["fp_ns_per_ray_row"] = res["fp_us"] * 1e3 / (a * detectors * size)
        res["bp_ns_per_pixel_angle"] = res["bp_us"] * 1e3 / (size * size * a)
        out[str(a)] = res
    return {"size": size, "detectors": detectors, "angles": out}


def run_warm(dev, n=64, per_image=16, tol=1e-3, max_iters=8000):
    """The headline comparison: milliseconds and iterations to relative
    residual 1e-3, plain zero-start SIRT against warm-started SIRT
    (warmstart.solve), on 64 held-out noise-free phantoms at N=256, 180
    angles, 363 detectors; the network is the committed checkpoint that this
    library trained on GPU-made pairs (its metadata is reported)."""
    import torch

    from synkrotomo_gb300 import warmstart
    from synkrotomo_gb300.unet import UNet
    if not os.path.exists(WARM_CHECKPOINT):
        return {"unavailable": f"checkpoint {os.path.relpath(WARM_CHECKPOINT, ROOT)} not found"}
    net = UNet(256, 32, seed=0)
    meta = net.load_checkpoint(WARM_CHECKPOINT)
    prob = warmstart.Problem(256, 180, noise=0.0)
    out = warmstart.headline(net, prob, n=n, seed=777777, tol=tol, max_iters=max_iters, per_image=per_image)
    out["checkpoint"] = {"file": os.path.relpath(WARM_CHECKPOINT, ROOT), **meta}
    del net
    torch.cuda.synchronize()
    return out


def unet_flops(size, batch):
    """Tensor-core FLOPs of one U-Net training step (2*H*W*Cin*Cout*9 per 3x3
    conv and pass): forward, backward-data and backward-weights of the 13
    convolutions on the tcgen05 engine (the Cin = 1 input conv runs on CUDA
    cores and is left out; its backward-data pass is not needed)."""
    from synkrotomo_gb300.unet import LAYERS
    level = [0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0]
    fwd = 0.0
    for (ci, co), lv in zip(LAYERS[1:], level[1:]):
        hw = (size >> lv) ** 2
        fwd += 2.0 * hw * batch * ci * co * 9
    return 3.0 * fwd


def run_unet(dev, size=256, batch=32, steps=10):
    """U-Net warm-starter training step (N=256, batch 32): ms per step and
    tensor-core TFLOP/s against the measured BF16 peak."""
    import torch

    from synkrotomo_gb300.unet import UNet

    net = UNet(size, batch, seed=0)
    g = torch.Generator(device=dev).manual_seed(0)
    x = torch.rand(batch, size, size, device=dev, generator=g)
    t = torch.rand(batch, size, size, device=dev, generator=g)
    for _ in range(3):
        net.train_step(x, t, lr=1e-4)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        net.train_step(x, t, lr=1e-4)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    fl = unet_flops(size, batch)
    e0.record()
    for _ in range(steps):
        net.forward(x)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / steps
    return {"size": size, "batch": batch, "ms_per_train_step": ms, "tflops_train": fl / (ms * 1e-3) / 1e12,
            "ms_forward": fwd_ms, "tflops_forward": fl / 3 / (fwd_ms * 1e-3) / 1e12,
            "tensor_flops_per_step": fl}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--legs", default=",".join(LEGS),
                    help="comma list of: proj (device-resident FP+BP, always run), e2e, sirt, csr, cpu, "
                         "batch (64 uneven problems), stack (slice stack)")
    ap.add_argument("--size", type=int, default=2048, help="image side (profiling cases; default: the benchmark)")
    ap.add_argument("--angles", type=int, default=2048)
    ap.add_argument("--detectors", type=int, default=0, help="0: ceil(size*sqrt(2))")
    args = ap.parse_args()
    args.legs = set(x.strip() for x in args.legs.split(",") if x.strip()) | {"proj"}
    set_workload(args.size, args.angles, args.detectors)
    args.warmup = max(3, args.warmup)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        # whole steps: every angle of the forward projection and of the
        # backprojection, W untimed, then K timed (no sampling, no scaling)
        r = None
        times, fps, bps = [], [], []
        for _ in range(args.warmup + args.steps):
            r = cpu_reference_step()
            times.append(r["step_s"])
            fps.append(r["fp_s"])
            bps.append(r["bp_s"])
        timed = times[args.warmup:]
        step_s = sum(timed) / len(timed)
        value = step_bytes() / step_s / 1e9
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": bench_config(args.gpus),
                "cpu_baseline": {"value": value, "unit": "GB/s", "cores": r["cores"], "kind": "port",
                                 "sample": f"whole steps: all {N_ANGLES} angles of FP and BP per step, mean of "
                                           f"{args.steps} after {args.warmup} untimed (oracle/cpu_ref.c, "
                                           f"{cpu_flags()}, {cpu_model()})"},
                "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "fp_ms": 1e3 * statistics.mean(fps[args.warmup:]), "bp_ms": 1e3 * statistics.mean(bps[args.warmup:])}
        print(json.dumps(line))
        return 0

    import torch
    if world > 1:
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    from synkrotomo_gb300 import _lib
    _lib.load()

    res = run_gpu(args, rank, world)
    if world > 1:
        torch.distributed.destroy_process_group()
    if rank != 0:
        return 0

    value = world * step_bytes() / (res["step_ms"] * 1e-3) / 1e9
    peaks = measured_peaks()
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    fp32_peak = res["sms"] * 128 * 2 * sm_max * 1e6 / 1e12     # TFLOP/s
    fp_tf = flops_fp() / (res["fp_ms"] * 1e-3) / 1e12
    bp_tf = flops_bp() / (res["bp_ms"] * 1e-3) / 1e12
    dom = "bp" if res["bp_ms"] >= res["fp_ms"] else "fp"
    achieved = bp_tf if dom == "bp" else fp_tf
    kname = "bp_tile_kernel" if dom == "bp" else "fp_lane_kernel"
    roofline = {"bound": "fp32", "kernel": kname, "achieved": achieved,
                "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                "traffic": None,
                "peak_source": f"nominal FP32: {res['sms']} SMs x 128 FMA/clk x 2 x {sm_max:.0f} MHz "
                               "(MEASURED_PEAKS.json has no FP32 figure)",
                "fp_tflops": fp_tf, "bp_tflops": bp_tf}
    line = {"metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["step_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world),
            "fp_ms": res["fp_ms"], "bp_ms": res["bp_ms"],
            # per step: setup (geometry_kernel when a > 1024, setup_kernel) + fp_lane_kernel + fp_exact_kernel
            # (FP); setup + row_scale_kernel + bp_tile_kernel (BP)
            "gpu_launches": (2 * (2 if N_ANGLES > 1024 else 1) + 4) * args.steps,
            "clocks": res["clocks"], "roofline": roofline}
    e = res["e2e"]
    if e is not None:
        line["e2e"] = {"value": world * step_bytes() / (e["ms"] * 1e-3) / 1e9, "unit": "GB/s",
                       "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"], "ms_per_step": e["ms"]}
    if res["sirt"] is not None:
        line["sirt_cfg0"] = res["sirt"]
    if res["csr"] is not None:
        c = res["csr"]
        hbm = float(peaks.get("hbm_gbs", 6800.0))
        for k in ("Ax", "ATy"):
            c[k]["frac_hbm"] = c[k]["GB/s"] / hbm
        c["hbm_peak_gbs"] = hbm
        line["csr_cfg1"] = c
    for key in ("batch", "stack", "sparse"):
        if res[key] is not None:
            line[{"batch": "sirt_batch_cfg3", "stack": "sirt_stack_cfg2", "sparse": "sparse_view"}[key]] = res[key]
    if res["unet"] is not None:
        u = res["unet"]
        bf16 = float(peaks.get("bf16_tflops", 1900.0))
        u["frac_train_of_measured_bf16"] = u["tflops_train"] / bf16
        u["frac_forward_of_measured_bf16"] = u["tflops_forward"] / bf16
        u["bf16_peak_tflops"] = bf16
        line["unet_cfg4"] = u
    if res["warm"] is not None:
        line["warm_start"] = res["warm"]
    if res["shard"] is not None:
        line["sirt3d_sharded"] = res["shard"]
    if "cpu" in args.legs:
        if "sirt_cfg0" in line:
            c0 = cpu_sirt_cfg0()
            line["sirt_cfg0"]["cpu_port_200_iterations_ms"] = c0["s"] * 1e3
            line["sirt_cfg0"]["cpu_port_cores"] = c0["cores"]
        r = cpu_reference_step()
        cv = step_bytes() / r["step_s"] / 1e9
        line["cpu_baseline"] = {"value": cv, "unit": "GB/s", "cores": r["cores"], "kind": "port",
                                "sample": f"one whole step (all {N_ANGLES} angles of FP and BP; oracle/cpu_ref.c, "
                                          f"{cpu_flags()}, {cpu_model()})"}
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
