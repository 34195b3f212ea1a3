"""bench.py's reference arm (CPU only): the JSON line it prints and the
silent exit of ranks other than 0.  A small workload keeps it to seconds; the
driver runs the full one."""
import json
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2", "--warmup", "3",
           "--size", "64", "--angles", "16"]
    return subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)


def test_reference_arm_line():
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 3
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    # whole steps, nothing scaled; the same config dict as the GPU arm prints
    assert "whole steps" in cb["sample"] and "scaled" not in cb["sample"]
    b = _bench_module()
    b.set_workload(64, 16, 0)
    assert d["config"] == b.bench_config(d["n_gpus"])


def test_reference_arm_other_ranks_print_nothing():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [l for l in r.stdout.splitlines() if l.startswith("{")]


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_summary_reads_the_samples_of_the_timed_region():
    bench = _bench_module()
    cs = bench.ClockSampler()
    # index, clocks.sm, clocks.max.sm, power, active mask, hw, hw_thermal, sw_thermal, sw_power_cap
    before = "0, 1200, 2070, 300.0, 0x0, Not Active, Not Active, Not Active, Not Active"
    inside = ["0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
              "0, 2040, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active",
              "0, 2055, 2070, 1100.0, 0x0, Not Active, Not Active, Not Active, Not Active"]
    cs.lines = [before] + inside
    cs.start = 1
    s = cs.summary()
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    cs.lines = [before, "0, 1900, 2070, 1300.0, 0x40, Not Active, Active, Not Active, Not Active"]
    cs.start = 1
    assert cs.summary()["reasons"] == ["hw_thermal_slowdown"]
    # a region too short for a sample: the last one before its end
    cs.lines, cs.start = [before], 1
    assert cs.summary()["sm_mhz"] == 1200.0
    cs.lines, cs.start = [], 0
    assert cs.summary()["reasons"] == ["unsampled"]


def test_bench_stack_generator_matches_phantom():
    """The bench's device-side slice-stack generator evaluates
    phantom.ellipsoid_volume's seeded ellipsoids with the same rule."""
    import bench
    import torch
    from synkrotomo_gb300 import phantom
    for size, ns, seed in ((32, 9, 3), (48, 12, 0)):
        got = bench._ellipsoid_stack_gpu(size, ns, seed, torch.device("cpu")).numpy()
        np.testing.assert_array_equal(got, phantom.ellipsoid_volume(size, ns, seed))
