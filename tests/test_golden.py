"""The committed golden fixtures (tests/golden/oracle_small.npz, written by
tests/golden/make_golden.py from the pinned oracles).

CPU: the oracles still give the committed numbers.  GPU: the CUDA path on the
committed inputs matches the committed FP32-oracle outputs within the parity
bar (1e-5 relative L2), and the FP64 ones where the two oracles agree."""
import importlib.util
import os

import numpy as np
import pytest
import torch

from tests.conftest import rel_l2

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "oracle_small.npz")


def _load():
    return np.load(FIXTURE)


def _maker():
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _prefixes(d, kind):
    return sorted({k.rsplit("_", 1)[0] for k in d.files if k.startswith(kind + "_")})


def test_oracles_reproduce_the_fixtures():
    d = _load()
    now = _maker().cases()
    assert sorted(now) == sorted(d.files)
    for k in d.files:
        a, b = now[k], d[k]
        assert a.shape == b.shape and a.dtype == b.dtype, k
        if k.endswith(("32", "64")):
            # float32 C oracle: libm's cosf/sinf may differ by an ulp between machines
            tol = 1e-6 if k.endswith("32") else 1e-12
            assert rel_l2(a, b) < tol, k
        else:
            np.testing.assert_array_equal(a, b, err_msg=k)


def _dev(x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.gpu
def test_cuda_projectors_match_the_fixtures(gpu):
    from synkrotomo_gb300 import runtime as rt
    d = _load()
    for p in _prefixes(d, "proj"):
        n, a, nr, rz, dr = d[p + "_geom"]
        n, nr = int(n), int(nr)
        ang = _dev(d[p + "_angles"])
        fp = rt.forwardprojection(ang, float(rz), float(dr), nr, _dev(d[p + "_image"])).cpu().numpy()
        bp = rt.backprojection(ang, float(rz), float(dr), n, _dev(d[p + "_sino"])).cpu().numpy()
        for out, key in ((fp, "_fp"), (bp, "_bp")):
            r32, r64 = d[p + key + "32"], d[p + key + "64"]
            assert rel_l2(out, r32) < 1e-5, p + key
            if rel_l2(r32, r64) < 1e-5:
                assert rel_l2(out, r64) < 1e-5, p + key


@pytest.mark.gpu
def test_cuda_sirt_matches_the_fixtures(gpu):
    from synkrotomo_gb300 import runtime as rt
    d = _load()
    for p in _prefixes(d, "sirt"):
        n, a, nr, rz, dr, its = d[p + "_geom"]
        n, its = int(n), int(its)
        x0 = torch.zeros(n * n, device="cuda")
        x = rt.sirt(_dev(d[p + "_angles"]), float(rz), float(dr), x0, _dev(d[p + "_sino"]), its).cpu().numpy()
        assert rel_l2(x, d[p + "_x32"]) < 1e-5, p
        assert rel_l2(x, d[p + "_x64"]) < 1e-4, p
