"""Restoration (Object::restorePatch with the Scharmer filter): the C restatement against an
independent numpy statement of the same steps (CPU only)."""
import numpy as np
import pytest

import oracle
from oracle import np_oracle
from tests.conftest import workload


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_restore_c_vs_numpy(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    op = oracle.OraclePatch(w.job)
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[0]
    op.set_images(w.patches.cutouts[0], None, fg)
    a = w.patches.alpha_true[0]
    fc = w.job.otf_size / 2.0
    filt = op.restore(a, fc)
    raw = op.restore(a, fc, no_filter=True)
    op.metric(a)
    D, S = op.D(), op.otf()
    noise = op.stats()[2]
    for o in range(w.job.n_objects):
        args = (D, S, noise, w.job.img_object, o, fc, w.job.patch_size, w.job.support.otf_support)
        ref = np_oracle.restore(*args)
        ref_raw = np_oracle.restore(*args, no_filter=True)
        # the filter's smoothing is summed directly in C and by an integral image in numpy
        assert np.abs(filt[o] - ref).max() <= 1e-9 * np.abs(ref).max()
        assert np.abs(raw[o] - ref_raw).max() <= 1e-12 * np.abs(ref_raw).max()


def test_smooth_window_is_the_references():
    # smooth(d, 1, 1) averages [y-1, y+1) x [x-1, x+1): the pixel and its upper/left neighbours
    d = np.arange(16.0).reshape(4, 4)
    s = np_oracle.smooth(d, 1, 1)
    assert s[0, 0] == 0.0
    assert s[1, 1] == (d[0, 0] + d[0, 1] + d[1, 0] + d[1, 1]) / 4
    assert s[3, 0] == (d[2, 0] + d[3, 0]) / 2


def test_restore_outputs_properties(w0):
    # the statement of the PSF, convolved-object and residual outputs: a PSF sums to the OTF
    # at zero frequency; the convolved object of a unit impulse at the origin is the
    # un-centred PSF; the residual of the convolved object is that minus the cutout image
    op = oracle.OraclePatch(w0.job)
    op.set_images(w0.patches.cutouts[0], None, w0.patches.fixed_gamma[0])
    a = w0.patches.alpha_true[0]
    op.metric(a)
    D, S = op.D(), op.otf()
    N, ps, I = w0.job.otf_size, w0.job.patch_size, w0.job.n_images
    obj = op.restore(a, N / 2.0)
    psf, psf_mean, cobj, res = np_oracle.restore_outputs(D, S, w0.job.img_object, obj, ps)
    for j in range(I):
        assert abs(psf[j].astype(np.float64).sum() - S[j, N // 2, N // 2].real) <= 1e-6 * abs(S[j, N // 2, N // 2])
    np.testing.assert_allclose(psf_mean[0], psf[w0.job.img_object == 0].astype(np.float64).mean(0),
                               rtol=0, atol=1e-6 * np.abs(psf).max())
    delta = np.zeros((1, N, N))
    delta[0, 0, 0] = 1.0
    _, _, cd, _ = np_oracle.restore_outputs(D, S, np.zeros(I, int), delta, ps)
    np.testing.assert_allclose(cd[0], np.fft.ifftshift(psf[0]), rtol=0, atol=1e-6 * np.abs(psf[0]).max())
    img = np.real(np.fft.ifft2(np.fft.ifftshift(D[0])))
    np.testing.assert_allclose(res[0], cobj[0].astype(np.float64) - img, rtol=0, atol=1e-3)
    # the image is the windowed, mean-padded cutout: its mean is the cutout mean
    assert abs(img.mean() - op.stats()[0][0]) <= 1e-6 * abs(op.stats()[0][0])
