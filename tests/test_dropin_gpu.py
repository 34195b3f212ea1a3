"""The ``futhark`` drop-in package, used exactly as the reference's README
(README.md:21-25) shows."""
import numpy as np
import pytest

from oracle import cpu_ref
from synkrotomo_gb300 import phantom
from tests.conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_readme_usage(gpu):
    from futhark import SIRT
    g = phantom.geometry(64, 60)
    img = phantom.ellipse_phantom(64, seed=9)
    sinogram = cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img).reshape(60, -1)
    theta = g.angles.astype(np.float64)
    emptyimage = np.zeros(64 * 64, np.float32)
    sirt = SIRT.SIRT()
    result = sirt.main(theta.astype(np.float32), g.rhozero, g.deltarho, emptyimage,
                       sinogram.flatten().astype(np.float32), 30).get()
    assert result.dtype == np.float32 and result.shape == (64 * 64,)
    reconstruction_result = result.reshape((64, 64))
    ref = cpu_ref.sirt(g.angles, g.rhozero, g.deltarho, emptyimage, sinogram.ravel(), 30)
    assert rel_l2(reconstruction_result.ravel(), ref) < 1e-5
    assert SIRT.SIRT.entry_points["main"][0][-1] == "i32"


def test_all_modules(gpu):
    from futhark import (SIRT3D, backprojection, backprojection_sparse, forwardprojection,
                         forwardprojection_sparse)
    g = phantom.geometry(32, 5)
    img = phantom.ellipse_phantom(32, seed=1)
    for cls in (forwardprojection.forwardprojection, forwardprojection_sparse.forwardprojection_sparse):
        s = cls().main(g.angles, g.rhozero, g.deltarho, g.numrhos, img).get()
        assert rel_l2(s, cpu_ref.forwardprojection(g.angles, g.rhozero, g.deltarho, g.numrhos, img)) < 1e-5
    y = np.random.default_rng(0).random(g.n_rays).astype(np.float32)
    for cls in (backprojection.backprojection, backprojection_sparse.backprojection_sparse):
        b = cls().main(g.angles, g.rhozero, g.deltarho, 32, y).get()
        assert rel_l2(b, cpu_ref.backprojection(g.angles, g.rhozero, g.deltarho, 32, y)) < 1e-5
    size = 8
    g8 = phantom.geometry(size, 4, numrhos=12)
    rhos = (g8.rhozero + np.arange(12)).astype(np.float32)
    proj = np.random.default_rng(1).random(size * 4 * 12).astype(np.float32)
    v = SIRT3D.SIRT3D().main(g8.angles, rhos, proj, 3, size).get()
    assert rel_l2(v, cpu_ref.sirt3d(g8.angles, rhos, proj, 3, size)) < 1e-5


def test_sirt3d_nslices_keyword(gpu):
    """A non-cubic stack: nslices slices of size x size (keyword without a
    reference counterpart), the same per-slice SIRT as the cubic call."""
    from futhark import SIRT3D
    size, a, ns, nr = 16, 10, 3, 24
    g = phantom.geometry(size, a, numrhos=nr)
    rhos = (g.rhozero + np.arange(nr)).astype(np.float32)
    proj = np.random.default_rng(4).random(ns * a * nr).astype(np.float32)
    v = SIRT3D.SIRT3D().main(g.angles, rhos, proj, 5, size, nslices=ns).get()
    assert v.shape == (ns * size * size,)
    assert rel_l2(v, cpu_ref.sirt3d(g.angles, rhos, proj, 5, size, nslices=ns)) < 1e-5
    with pytest.raises(ValueError):
        SIRT3D.SIRT3D().main(g.angles, rhos, proj, 5, size, nslices=ns + 1)


def test_argument_errors(gpu):
    from futhark import SIRT, backprojection, forwardprojection
    g = phantom.geometry(16, 4)
    img = np.zeros(256, np.float32)
    fp = forwardprojection.forwardprojection()
    with pytest.raises(TypeError):
        fp.main(g.angles.astype(np.float64), g.rhozero, g.deltarho, g.numrhos, img)
    with pytest.raises(TypeError):
        fp.main(g.angles, g.rhozero, g.deltarho, 2.5, img)
    with pytest.raises(ValueError):
        fp.main(g.angles, g.rhozero, g.deltarho, g.numrhos, np.zeros(250, np.float32))   # not square
    with pytest.raises(ValueError):
        fp.main(g.angles, g.rhozero, g.deltarho, g.numrhos, np.zeros(225, np.float32))   # odd side
    with pytest.raises(ValueError):
        fp.main(np.zeros(0, np.float32), g.rhozero, g.deltarho, g.numrhos, img)        # no angles
    with pytest.raises(ValueError):
        backprojection.backprojection().main(g.angles, g.rhozero, g.deltarho, 16, np.zeros(10, np.float32))
    with pytest.raises(ValueError):
        fp.main(g.angles, g.rhozero, 0.0, g.numrhos, img)                                # deltarho 0
    with pytest.raises(ValueError):
        SIRT.SIRT().main(g.angles, g.rhozero, g.deltarho, img, np.zeros(g.n_rays, np.float32), -1)
