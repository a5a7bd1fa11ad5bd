"""FIT_PLANE (the RF_FIT_PLANE run flag): the plane fitted to each object's mean image is
removed inside the window before the transforms, refitted after re-shifts and added back to
the restored object (Object::fitAvgPlane, object.cpp:553-594; SubImage::getWindowedImg,
subimage.cpp:106-150; Object::restorePatch, object.cpp:410-413).  The oracle is checked
against a numpy statement on the CPU; the GPU against the oracle (marked gpu)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import jobsetup as js
from redux_gb300 import solver as S
from tests.conftest import workload


def _oracle(w, p=0, plane=True):
    op = oracle.OraclePatch(w.job)
    op.set_fit_plane(plane)
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[p]
    op.set_images(w.patches.cutouts[p], None, fg)
    return op


def _np_plane(job, cut):
    """The mean image of each object (float sums in image order, float division), its
    least-squares plane without the constant, rounded to float."""
    ps = job.patch_size
    m = (job.cutout_size - ps) // 2
    yy, xx = np.mgrid[0:ps, 0:ps]
    out = []
    for o in range(job.n_objects):
        idx = [j for j in range(job.n_images) if job.img_object[j] == o]
        acc = np.zeros((ps, ps), np.float32)
        for j in idx:
            acc = (acc + cut[j, m:m + ps, m:m + ps]).astype(np.float32)
        avg = (acc / np.float32(len(idx))).astype(np.float32)
        coef, _ = js.fit_plane(avg.astype(np.float64), np.ones((ps, ps)))
        out.append((coef[0] * (yy - ps // 2) + coef[1] * (xx - ps // 2)).astype(np.float32))
    return np.stack(out)


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_oracle_plane_is_the_least_squares_plane(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=1, frames=4)
    op = _oracle(w)
    ref = _np_plane(w.job, w.patches.cutouts[0])
    np.testing.assert_allclose(op.plane(), ref, rtol=0, atol=1e-6 * np.abs(ref).max())
    assert np.abs(ref).max() > 1.0     # the synthetic images do have a slope


def test_oracle_image_transform_removes_the_plane(w0):
    job, cut = w0.job, w0.patches.cutouts[0]
    op = _oracle(w0)
    pl = op.plane()
    ps = job.patch_size
    m = (job.cutout_size - ps) // 2
    for j in range(job.n_images):
        img = cut[j, m:m + ps, m:m + ps].astype(np.float64)
        avg = img.mean()
        win = (img - avg - pl[job.img_object[j]]) * job.window + avg
        D = np.fft.fftshift(np.fft.fft2(win))
        np.testing.assert_allclose(op.D()[j], D, rtol=0, atol=1e-9 * np.abs(D).max())


gpu = pytest.mark.gpu
TOL_METRIC = 1e-5
TOL_RESTORE = 1e-4


def _solver(w):
    s = S.Solver(w.job, max_patches=w.patches.cutouts.shape[0])
    s.set_fit_plane(True)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return s


@gpu
@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_image_transform_metric_and_restore(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    D = s.debug("D")
    a = w.patches.alpha_true * 0.5
    L = s.metric(a)
    fc = w.job.otf_size / 2.0
    obj = s.restore(a, fc)
    for p in range(a.shape[0]):
        op = _oracle(w, p)
        Do = op.D()
        assert np.linalg.norm(D[p] - Do) / np.linalg.norm(Do) < 1e-6
        Lo = op.metric(a[p])
        assert abs(L[p] - Lo) <= TOL_METRIC * abs(Lo), (p, L[p], Lo)
        ref = op.restore(a[p], fc)
        for o in range(w.job.n_objects):
            err = np.abs(obj[p, o] - ref[o]).max() / np.abs(ref[o]).max()
            assert err <= TOL_RESTORE, (p, o, err)
    # switching the plane off prepares the images again without it
    s.set_fit_plane(False)
    op0 = _oracle(w, 0, plane=False)
    assert abs(s.metric(a)[0] - op0.metric(a[0])) <= TOL_METRIC * abs(op0.metric(a[0]))


@gpu
def test_staged_solve_refits_after_reshifts(w0):
    """Two mode stages with a re-shift between them: the planes are refitted to the re-cut
    images before they are prepared again, on the GPU as in the oracle."""
    job = w0.job
    kw = dict(max_iterations=3, min_iterations=3, ftol=1e-3)
    s = _solver(w0)
    out = s.run(S.SolveSettings(mode_start=5, mode_step=job.n_modes, max_metrics=64, **kw))
    op = _oracle(w0)
    ref = op.solve(oracle.Cfg(n_initial_modes=5, n_mode_increment=job.n_modes, target_iterations=3, fd_first=1,
                              eps=1e-10, brent_tol=0.1, **kw))
    assert out["reports"][0].iterations == ref["report"].iterations
    np.testing.assert_allclose(out["metrics"][0, :3], ref["metrics"][:3], rtol=1e-5)
    sg, so = s.debug("shifts")[0], op.shifts()[0]
    assert np.any(so != 0)
    np.testing.assert_array_equal(sg, so)
    # after the re-shift: the image transforms of the re-cut images with the refitted planes
    Dg, Do = s.debug("D")[0], op.D()
    assert np.linalg.norm(Dg - Do) / np.linalg.norm(Do) < 1e-6
