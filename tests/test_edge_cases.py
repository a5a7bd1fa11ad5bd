"""Edge cases of the boundary: arguments rdxg_create rejects before it touches a device (CPU),
and on the GPU an object of weight zero, an image without variance, a batch smaller than the
handle's capacity and the smallest compiled size, each against the FP64 oracle."""
import dataclasses

import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S
from redux_gb300 import synth
from tests.conftest import workload


def _job32():
    return synth.make_job(32, 10, synth.LAYOUT_1OBJ(2))


@pytest.mark.parametrize("change, status, msg", [
    (dict(otf_size=40), 1, "otf_size must be 2 \\* pupil_pixels"),
    (dict(otf_size=48, pupil_pixels=24, patch_size=48), 2, "otf_size not compiled"),
    (dict(patch_size=30), 2, "patch_size must equal otf_size"),
])
def test_create_rejects_bad_geometry(change, status, msg):
    job = dataclasses.replace(_job32(), **change)
    with pytest.raises(S.SolverError, match=f"status {status}: {msg}"):
        S.Solver(job, max_patches=1)


def test_create_rejects_objects_whose_images_are_not_contiguous():
    job = _job32()
    io = job.img_object.copy()
    io[1], io[-1] = 1, 0          # object 0, object 1, ..., object 0
    job2 = dataclasses.replace(job, img_object=io, obj_weight=np.ones(2), obj_grad_step=np.ones(2))
    with pytest.raises(S.SolverError, match="status 1: images of an object must be contiguous"):
        S.Solver(job2, max_patches=1)


gpu = pytest.mark.gpu


def _oracle(job, cut, fg=None):
    op = oracle.OraclePatch(job)
    op.set_images(cut, None, fg)
    return op


@gpu
def test_object_of_weight_zero():
    """Object::weight 0 drops the object from the metric and zeroes its gradient
    (solver.cpp:763-817, 881)."""
    w = workload("production88", n_patches=1, frames=4)
    job = dataclasses.replace(w.job, obj_weight=np.array([1.0, 0.0]))
    s = S.Solver(job, max_patches=1)
    s.set_patches(w.patches.cutouts)
    a = w.patches.alpha_true * 0.5
    op = _oracle(job, w.patches.cutouts[0])
    L = s.metric(a)[0]
    assert abs(L - op.metric(a[0])) <= 1e-5 * abs(op.metric(a[0]))
    g, _ = s.gradient(a, "vogel")
    _, go = op.gradient(a[0], method="vogel")
    obj1 = job.img_object == 1
    assert np.all(g[0][obj1] == 0.0)
    assert np.linalg.norm(g[0] - go) / np.linalg.norm(go) < 1e-5


@gpu
def test_image_without_variance_is_reported():
    """A constant image has no noise estimate relative to its spread: the noise-derived
    regularisation is not finite and set_patches answers RDXG_ERR_NONFINITE."""
    w = workload("plain64")
    cut = w.patches.cutouts.copy()
    cut[0, 1] = 1000.0
    s = S.Solver(w.job, max_patches=1)
    with pytest.raises(S.SolverError, match="status 5"):
        s.set_patches(cut)


@gpu
def test_batch_smaller_than_the_capacity():
    w = workload("production88", n_patches=2, frames=4)
    s = S.Solver(w.job, max_patches=3)
    a = w.patches.alpha_true * 0.5
    s.set_patches(w.patches.cutouts[1:2])
    L1 = s.metric(a[1:2])
    s.set_patches(w.patches.cutouts)
    L2 = s.metric(a)
    for p, L in ((1, L1[0]), (0, L2[0]), (1, L2[1])):
        Lo = _oracle(w.job, w.patches.cutouts[p]).metric(a[p])
        assert abs(L - Lo) <= 1e-5 * abs(Lo), (p, L, Lo)
    with pytest.raises(S.SolverError, match="n_patches out of range"):
        s.set_patches(np.concatenate([w.patches.cutouts] * 2))


@gpu
def test_smallest_size_32():
    job = _job32()
    pt = synth.make_patches(job, 1, 8.0, np.random.default_rng(32))
    s = S.Solver(job, max_patches=1)
    s.set_patches(pt.cutouts)
    op = _oracle(job, pt.cutouts[0])
    a = pt.alpha_true * 0.5
    assert abs(s.metric(a)[0] - op.metric(a[0])) <= 1e-5 * abs(op.metric(a[0]))
    g, _ = s.gradient(a, "vogel")
    _, go = op.gradient(a[0], method="vogel")
    assert np.linalg.norm(g[0] - go) / np.linalg.norm(go) < 1e-5
    # the first iteration as the FP64 solver takes it (its line search then sees metric
    # changes near the FP32 rounding of this small problem, and the histories part)
    out = s.run(S.fixed_iterations(job.n_modes, 3, max_metrics=16))
    ref = op.solve(oracle.default_cfg(max_iterations=3, n_modes=job.n_modes))
    np.testing.assert_allclose(out["metrics"][0, :2], ref["metrics"][:2], rtol=1e-5)


@gpu
def test_full_batch_patches_are_independent():
    """At the production size (225 patches 88x88, 3 channels x 12 frames): a patch's solve does
    not depend on the other patches of its batch (the same bits as a 5-patch batch of some of
    them), and every patch ends below its initial metric."""
    w = workload("production88")
    P = w.patches.cutouts.shape[0]
    st = S.fixed_iterations(w.job.n_modes, 20, max_metrics=32)
    big = S.Solver(w.job, max_patches=P)
    big.set_patches(w.patches.cutouts)
    ob = big.run(st)
    big.close()
    idx = [0, 57, 112, 180, P - 1]
    small = S.Solver(w.job, max_patches=len(idx))
    small.set_patches(w.patches.cutouts[idx])
    osm = small.run(st)
    small.close()
    np.testing.assert_array_equal(ob["alpha"][idx], osm["alpha"])
    np.testing.assert_array_equal(ob["metrics"][idx], osm["metrics"])
    assert all(r.final_metric < r.initial_metric for r in ob["reports"])
