"""The validation programs (futhark/tools/*.fut) on the GPU against their
restatement, and the executable / futhark-bench harness end to end."""
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import fut_ref

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _pair(n, seed, scale=0.05):
    rng = np.random.default_rng(seed)
    s = rng.random(n).astype(np.float32)
    t = (s + rng.normal(0, scale, n)).astype(np.float32)
    return s, t


@pytest.mark.parametrize("n", [1, 2, 3, 1000, 1 << 20, (1 << 22) + 7])
def test_tools_match_restatement(gpu, n):
    from futhark.tools import diff, mse, sanityCheck
    s, t = _pair(n, n)
    t[0] = s[0] + 1.0          # index 0 is never counted by diff.fut
    d = diff.diff().main(s, t)
    assert isinstance(d, np.int32) and d == fut_ref.tools_diff(s, t)
    m = mse.mse().main(s, t)
    assert isinstance(m, np.float32)
    assert abs(float(m) - fut_ref.tools_mse(s, t)) <= 1e-6 * fut_ref.tools_mse(s, t)
    ok = sanityCheck.sanityCheck().main(s, t)
    assert bool(ok) == fut_ref.tools_sanity(s, t) == False


def test_tools_edge_cases(gpu):
    import torch
    from synkrotomo_gb300 import runtime as rt
    s = np.zeros(9, np.float32)
    t = s.copy()
    assert rt.compare(torch.from_numpy(s).cuda(), torch.from_numpy(t).cuda()) == (0, 0.0, True)
    t[4] = np.nan                          # a NaN is neither counted nor accepted
    cnt, sse, ok = rt.compare(torch.from_numpy(s).cuda(), torch.from_numpy(t).cuda())
    assert cnt == fut_ref.tools_diff(s, t) == 0 and not ok and not fut_ref.tools_sanity(s, t)
    t[4] = 0.05                            # exactly std_dev: not > and not <
    cnt, _, ok = rt.compare(torch.from_numpy(s).cuda(), torch.from_numpy(t).cuda())
    assert cnt == fut_ref.tools_diff(s, t) and ok == fut_ref.tools_sanity(s, t)
    # unaligned views take the scalar path
    big_s, big_t = _pair(4099, 7, 0.1)
    gs, gt = torch.from_numpy(big_s).cuda(), torch.from_numpy(big_t).cuda()
    cnt, sse, ok = rt.compare(gs[1:], gt[1:])
    assert cnt == fut_ref.tools_diff(big_s[1:], big_t[1:])
    assert abs(sse / 4098 - fut_ref.tools_mse(big_s[1:], big_t[1:])) < 1e-9
    empty = torch.empty(0, device="cuda")
    assert rt.compare(empty, empty) == (0, 0.0, True)
    from futhark.tools import diff
    with pytest.raises(ValueError):
        diff.diff().main(np.zeros(3, np.float32), np.zeros(4, np.float32))
    with pytest.raises(TypeError):
        diff.diff().main(np.zeros(3, np.float64), np.zeros(3, np.float32))


def test_executable_and_bench_harness(gpu, tmp_path):
    """python -m futhark.forwardprojection < dataset, and fbench over two
    generated datasets: same result as the library call, CSV in N;us form."""
    from synkrotomo_gb300 import fbench, fvalues
    from futhark import forwardprojection
    paths = []
    for n in (64, 96):
        p = str(tmp_path / f"fpinputf32rad{n}")
        fbench.generate("forwardprojection", n, p, n_angles=48, seed=n)
        paths.append(p)
    r = subprocess.run([sys.executable, "-m", "futhark.forwardprojection", "-r", "3", "-t",
                        str(tmp_path / "rt.txt"), "-b", "-i", paths[0]], cwd=ROOT, capture_output=True)
    assert r.returncode == 0, r.stderr.decode()[-2000:]
    (out,) = fvalues.read_values(r.stdout)
    args = fbench.parse_args_for("forwardprojection", fvalues.read_file(paths[0]))
    want = forwardprojection.forwardprojection().main(*args).get()
    np.testing.assert_array_equal(out, want)
    times = (tmp_path / "rt.txt").read_text().split()
    assert len(times) == 3 and all(int(x) > 0 for x in times)
    rows = fbench.bench("forwardprojection", paths, runs=3)
    assert [r[0] for r in rows] == [64, 96] and all(r[1] > 0 for r in rows)
    fbench.write_csv(rows, str(tmp_path / "fut_fp.csv"))
    lines = (tmp_path / "fut_fp.csv").read_text().splitlines()
    assert lines[0].startswith("64;") and lines[1].startswith("96;")
    # a dataset with a wrong type is rejected like the compiled program does
    bad = tmp_path / "bad"
    bad.write_text("[0.0f32] 1.0f32 1.0f32 4.0f32 [0.0f32, 0.0f32, 0.0f32, 0.0f32]")
    r = subprocess.run([sys.executable, "-m", "futhark.forwardprojection", "-i", str(bad)], cwd=ROOT,
                       capture_output=True)
    assert r.returncode == 1 and b"argument #3" in r.stderr
