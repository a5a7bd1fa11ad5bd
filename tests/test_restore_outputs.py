"""PSF, convolved-object and residual outputs of the restoration (rdxg_restore_ex) against the
numpy statement of Object::restorePatch's outputs on the FP64 oracle's OTFs and image
transforms at the same alpha (marked gpu).  The convolutions use the device's own restored
object (compared with the oracle's in test_gpu_parity), so the comparison isolates the PSF
and convolution arithmetic."""
import numpy as np
import pytest

import oracle
from oracle import np_oracle
from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu

# FP32 handles: OTFs and image transforms enter in FP32 (1e-7 of their peak), the outputs
# are computed in FP64 and stored as float
TOL = {"fp32": 2e-6, "fp64": 1e-7}


def _setup(cfg, precision):
    w = {"plain64": lambda: workload("plain64"),
         "production88": lambda: workload("production88", n_patches=2, frames=4),
         "large128": lambda: workload("large128", n_patches=1, frames=2)}[cfg]()
    P = w.patches.cutouts.shape[0]
    s = S.Solver(w.job, max_patches=P, precision=precision)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return w, s


def _oracle_outputs(w, p, a, objects):
    op = oracle.OraclePatch(w.job)
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[p]
    op.set_images(w.patches.cutouts[p], None, fg)
    op.metric(a)
    return np_oracle.restore_outputs(op.D(), op.otf(), w.job.img_object, objects, w.job.patch_size)


@pytest.mark.parametrize("cfg,precision", [("plain64", "fp32"), ("plain64", "fp64"), ("production88", "fp32"),
                                           ("large128", "fp32")])
def test_psf_cobj_residual(cfg, precision):
    w, s = _setup(cfg, precision)
    a = w.patches.alpha_true * 0.8
    fc = w.job.otf_size / 2.0
    out = s.restore_outputs(a, fc, psf="each", cobj=True, residual=True)
    ref_obj = s.restore(a, fc)
    np.testing.assert_array_equal(out["objects"], ref_obj)
    tol = TOL[precision]
    for p in range(a.shape[0]):
        psf, _, cobj, res = _oracle_outputs(w, p, a[p], out["objects"][p])
        for name, got, ref in (("psf", out["psf"][p], psf), ("cobj", out["cobj"][p], cobj)):
            err = np.abs(got - ref).max() / np.abs(ref).max()
            assert err <= tol, (name, p, err)
        # the residual is a small difference of image-sized values: measured on their scale
        err = np.abs(out["residual"][p] - res).max() / np.abs(cobj).max()
        assert err <= tol, ("residual", p, err)


def test_psf_mean():
    w, s = _setup("production88", "fp32")
    a = w.patches.alpha_true * 0.8
    fc = w.job.otf_size / 2.0
    each = s.restore_outputs(a, fc, psf="each")["psf"]
    mean = s.restore_outputs(a, fc, psf="mean")["psf"]
    for p in range(a.shape[0]):
        _, psf_mean, _, _ = _oracle_outputs(w, p, a[p], np.zeros((w.job.n_objects, w.job.otf_size, w.job.otf_size)))
        for o in range(w.job.n_objects):
            sel = w.job.img_object == o
            np.testing.assert_allclose(mean[p, o], each[p, sel].astype(np.float64).mean(0), rtol=0,
                                       atol=1e-6 * np.abs(each[p, sel]).max())
            err = np.abs(mean[p, o] - psf_mean[o]).max() / np.abs(psf_mean[o]).max()
            assert err <= TOL["fp32"], (p, o, err)


def test_flag_errors():
    from redux_gb300 import _lib
    w, s = _setup("plain64", "fp32")
    a = np.ascontiguousarray(w.patches.alpha_true, np.float64)
    fc = np.full(w.job.n_objects, 16.0)
    obj = np.zeros((1, w.job.n_objects, w.job.patch_size, w.job.patch_size), np.float32)
    L = _lib.load()
    # a PSF requested without a buffer, an unknown flag
    assert L.rdxg_restore_ex(s.h, _lib.ptr(a), _lib.ptr(fc), 0, _lib.RDXG_RESTORE_PSF, _lib.ptr(obj),
                             None, None, None) == _lib.RDXG_ERR_ARG
    assert L.rdxg_restore_ex(s.h, _lib.ptr(a), _lib.ptr(fc), 0, 16, _lib.ptr(obj), None, None, None) == _lib.RDXG_ERR_ARG
