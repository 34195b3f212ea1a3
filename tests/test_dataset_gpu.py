"""The reference's own dataset, futhark/data/fpinputf32rad512, through the
drop-in programs on the GPU (its exact copy: tests/golden/fpinputf32rad512.npz).

The dataset is forwardprojection.main's input as the reference benchmarks it
(futhark/forwardprojection.fut:1-14): 805 angles in [pi/4, 3pi/4) (all flat
lines; the first one, f32(pi/4), sits on the steep/flat boundary), rhozero
-362, deltarho 1, 725 detectors and a 512 x 512 image of 10 grey levels.  The
reference ships no expected output for it, so the checks are against the
FP32 restatement and the FP64 restatement on sampled angles and rows, both
at 1e-5 relative L2 (on this dataset the two restatements agree to 2.4e-6
(forward) and 7.4e-7 (backward), so both bars apply).
"""
import numpy as np
import pytest

from oracle import cpu_ref
from oracle import fut_ref as F
from tests.conftest import load_fpinput512, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _both_oracles(gpu_part, f32_part, f64_part):
    assert rel_l2(f32_part, f64_part) < TOL        # the oracles agree here
    assert rel_l2(gpu_part, f64_part) < TOL


def test_forwardprojection_main_on_the_reference_dataset(gpu):
    from futhark import forwardprojection
    angles, rz, dr, nr, img = load_fpinput512()
    got = forwardprojection.forwardprojection().main(angles, rz, dr, nr, img).get()
    assert got.shape == (805 * 725,) and got.dtype == np.float32
    ref32 = cpu_ref.forwardprojection(angles, rz, dr, nr, img)
    assert rel_l2(got, ref32) < TOL
    assert np.max(np.abs(got - ref32)) <= 1e-4 * float(np.max(np.abs(ref32)))
    # FP64 on 41 angles: both ends, the two next to pi/2, and an even spread
    idx = np.unique(np.r_[0, 1, 401, 402, 403, 404, 804, np.linspace(0, 804, 37).astype(int)])
    ref64 = F.forwardprojection(angles[idx], rz, dr, nr, img).reshape(idx.size, nr)
    _both_oracles(got.reshape(805, nr)[idx], ref32.reshape(805, nr)[idx], ref64)
    # the sparse-view program is the same program (forwardprojection_sparse.fut:26-40)
    from futhark import forwardprojection_sparse
    got_s = forwardprojection_sparse.forwardprojection_sparse().main(angles, rz, dr, nr, img).get()
    np.testing.assert_array_equal(got_s, got)


def test_backprojection_main_on_the_reference_dataset(gpu):
    """backprojection.main on the dataset's geometry, fed the dataset's own
    sinogram (the FP32 restatement's forward projection of its image)."""
    from futhark import backprojection
    angles, rz, dr, nr, img = load_fpinput512()
    sino = cpu_ref.forwardprojection(angles, rz, dr, nr, img)
    got = backprojection.backprojection().main(angles, rz, dr, np.int32(512), sino).get()
    assert got.shape == (512 * 512,)
    ref32 = cpu_ref.backprojection(angles, rz, dr, 512, sino)
    assert rel_l2(got, ref32) < TOL
    assert np.max(np.abs(got - ref32)) <= 1e-4 * float(np.max(np.abs(ref32)))
    rows = [0, 1, 100, 255, 256, 411, 510, 511]
    ref64 = F.backprojection_rows(angles, rz, dr, 512, sino, rows)
    _both_oracles(got.reshape(512, 512)[rows], ref32.reshape(512, 512)[rows], ref64)


def test_sirt_main_on_the_reference_dataset(gpu):
    """SIRT.main on the dataset's geometry and sinogram, 10 iterations from a
    zero image, against the FP32 restatement (the 1e-5 plain-SIRT bar; 10
    iterations keep the CPU restatement's share of the test near 15 s)."""
    from futhark import SIRT
    angles, rz, dr, nr, img = load_fpinput512()
    sino = cpu_ref.forwardprojection(angles, rz, dr, nr, img)
    x0 = np.zeros(512 * 512, np.float32)
    got = SIRT.SIRT().main(angles, rz, dr, x0, sino, np.int32(10)).get()
    ref32 = cpu_ref.sirt(angles, rz, dr, x0, sino, 10)
    assert rel_l2(got, ref32) < TOL
    # the reconstruction approaches the dataset's image
    assert rel_l2(got, img) < 0.6
