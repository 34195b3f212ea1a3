"""Host-side argument handling of the runtime (CPU only: the library call is
replaced by a recorder)."""
import numpy as np
import pytest
import torch

from synkrotomo_gb300 import runtime as rt


def test_sirt3d_nslices_passes_the_stack_geometry(monkeypatch):
    seen = {}

    def record(angles, rhozero, deltarho, numrhos, size, nslices, image, projections, iterations, out=None, **kw):
        seen.update(rhozero=rhozero, deltarho=deltarho, numrhos=numrhos, size=size, nslices=nslices, image=image,
                    values=projections.numel(), iterations=iterations)
        return torch.zeros(nslices * size * size), None, None

    monkeypatch.setattr(rt, "sirt_slices", record)
    ang = torch.zeros(10)
    rhos = torch.from_numpy(np.float32(-11.5) + np.arange(24, dtype=np.float32))
    x = rt.sirt3d(ang, rhos, torch.zeros(3 * 10 * 24), 5, 16, nslices=3)
    assert x.shape == (3 * 16 * 16,)
    assert seen == dict(rhozero=-11.5, deltarho=1.0, numrhos=24, size=16, nslices=3, image=None, values=720,
                        iterations=5)
    with pytest.raises(ValueError):
        rt.sirt3d(ang, rhos, torch.zeros(3 * 10 * 24), 5, 16, nslices=0)
    with pytest.raises(ValueError):
        rt.sirt3d(ang, rhos, torch.zeros(3 * 10 * 24), 5, 16, nslices=4)     # stack length mismatch
    with pytest.raises(ValueError):
        rt.sirt3d(ang, rhos[:1], torch.zeros(30), 5, 16, nslices=3)          # one detector position


def test_detector_coverage_warning():
    import warnings as w
    from synkrotomo_gb300 import dropin
    with pytest.warns(dropin.DetectorCoverageWarning):
        assert dropin.check_detector_coverage(30, 1.0, 48, "backprojection")      # 30 < ceil(48*sqrt 2) = 68
    with pytest.warns(dropin.DetectorCoverageWarning):
        assert dropin.check_detector_coverage(136, 0.5, 96, "SIRT")               # 68 < 136
    with w.catch_warnings():
        w.simplefilter("error")
        assert not dropin.check_detector_coverage(68, 1.0, 48, "backprojection")  # the default row
        assert not dropin.check_detector_coverage(100, 1.0, 48, "backprojection")
        assert not dropin.check_detector_coverage(10, 0.0, 48, "SIRT")            # invalid: the library rejects it


class _FakeLib:
    """Stands in for libsynk: a context whose last call failed with ``rc``."""

    def __init__(self, rc, msg):
        self.rc, self.msg = rc, msg

    def synk_context_sync(self, handle):
        return self.rc

    def synk_context_get_error(self, handle):
        return self.msg.encode()


def _fake_context(rc, msg):
    ctx = object.__new__(rt._Context)
    ctx.handle, ctx.device, ctx.lib = None, 0, _FakeLib(rc, msg)
    return ctx


def test_timeout_status_reaches_the_caller():
    """A grid barrier that gave up leaves SYNK_ETIMEOUT in the context; the
    next sync raises it with the library's message (the failure is made by a
    fake of the library, no GPU involved)."""
    from synkrotomo_gb300 import _lib
    ctx = _fake_context(_lib.SYNK_ETIMEOUT, "persistent SIRT kernel: grid barrier timed out")
    with pytest.raises(rt.SynkError) as e:
        ctx.sync()
    assert e.value.code == _lib.SYNK_ETIMEOUT and "timed out" in str(e.value)
    with pytest.raises(ValueError):
        _fake_context(_lib.SYNK_EINVAL, "bad argument").check(_lib.SYNK_EINVAL, "call")
    _fake_context(0, "").sync()        # status 0: no exception
