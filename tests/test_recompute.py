"""Recomputed transforms (rdxg_set_recompute): the gradient kernels form the pupil function, its
transform X and (on the fused FP32 path) the OTF again from the phases instead of keeping them
per image, as the reference keeps SubImage::PF / SubImage::OTF (subimage.hpp:156-158) for
calcVogelWeight (subimage.cpp:348-371).  Gradients, finite-difference gradients, solves and
restorations with and without it, the automatic choice under a memory budget, and the
adjoint-check workload against the FP64 oracle with it on (marked gpu)."""
import os

import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu

# the fused path recomputes X and S with another transform order than the evaluation's
# half-plane form: rounding differences only
TOL_FUSED = 2e-6


def _solver(w, precision="fp32", P=None, recompute=None):
    P = w.patches.cutouts.shape[0] if P is None else P
    s = S.Solver(w.job, max_patches=P, precision=precision)
    if recompute is not None:
        s.set_recompute(recompute)
    s.set_patches(w.patches.cutouts[:P], None, None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[:P])
    return s


def _general(w, precision="fp32"):
    os.environ["RDXG_NO_FUSED"] = "1"
    try:
        return _solver(w, precision)
    finally:
        del os.environ["RDXG_NO_FUSED"]


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
@pytest.mark.parametrize("method", ["vogel", "exact", "fd"])
def test_fused_gradients_recomputed(cfg, method):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    assert not s.recompute()
    a = w.patches.alpha_true * 0.6
    g0, L0 = s.gradient(a, method)
    s.set_recompute(True)
    assert s.recompute()
    g1, L1 = s.gradient(a, method)
    assert _rel(g1, g0) < TOL_FUSED, _rel(g1, g0)
    np.testing.assert_allclose(L1, L0, rtol=1e-7)
    # and against the FP64 oracle (the finite-difference gradient to its own bound)
    if method == "vogel":
        for p in range(a.shape[0]):
            op = oracle.OraclePatch(w.job)
            op.set_images(w.patches.cutouts[p], None, None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[p])
            _, go = op.gradient(a[p], "vogel")
            assert _rel(g1[p], go) < 1e-5


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("method", ["vogel", "fd"])
def test_general_path_recomputed_bit_for_bit(precision, method):
    """On the general path the kept S is read as before and PF, X are formed by the same
    arithmetic as the evaluation's: the gradients are the same bits."""
    w = workload("plain64")
    s = _general(w, precision)
    a = w.patches.alpha_true * 0.6
    g0, _ = s.gradient(a, method)
    s.set_recompute(True)
    g1, _ = s.gradient(a, method)
    np.testing.assert_array_equal(g1, g0)


def test_general_path_n128_recomputed():
    w = workload("large128", n_patches=1, frames=2)
    s = _solver(w)
    a = w.patches.alpha_true * 0.5
    g0, _ = s.gradient(a, "vogel")
    s.set_recompute(True)
    g1, _ = s.gradient(a, "vogel")
    np.testing.assert_array_equal(g1, g0)


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_solve_recomputed(cfg):
    """A short solve (finite-difference first gradient, then Vogel) with recomputed transforms
    takes the same steps as with kept ones up to the gradient's rounding."""
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    st = S.fixed_iterations(w.job.n_modes, 4, max_metrics=64)
    r0 = _solver(w).run(st)
    r1 = _solver(w, recompute=True).run(st)
    for p in range(len(r0["reports"])):
        m0 = r0["metrics"][p, :3]
        m1 = r1["metrics"][p, :3]
        np.testing.assert_allclose(m1, m0, rtol=1e-6)
        assert r1["reports"][p].iterations == r0["reports"][p].iterations


def test_restore_recomputed():
    w = workload("production88", n_patches=2, frames=4)
    fc = w.job.otf_size / 2.0
    a = w.patches.alpha_true
    o0 = _solver(w).restore(a, fc)
    s1 = _solver(w, recompute=True)
    n0 = int(s1.debug("allocations")[0])
    o1 = s1.restore(a, fc)
    # the OTFs are held only during the call
    assert int(s1.debug("allocations")[0]) - n0 <= 5      # the restoration's own buffers (first call)
    np.testing.assert_allclose(o1, o0, rtol=0, atol=1e-6 * np.abs(o0).max())
    with pytest.raises(S.SolverError, match="not kept"):
        s1.debug("otf")


def test_memory_budget_selects_recompute():
    w = workload("production88", n_patches=2, frames=4)
    # generous budget: kept
    job = w.job
    os.environ["RDXG_MEMORY_BUDGET"] = str(1 << 40)
    try:
        s = S.Solver(job, max_patches=64)
        assert not s.recompute()
        total = int(s.debug("allocated_bytes")[0])
        s.close()
        # a budget that holds everything but half of the kept transforms (X, PF and the OTF of
        # every image; the recomputation's scratch is far smaller)
        N, n, I = job.otf_size, job.pupil_pixels, job.n_images
        kept = 64 * I * 8 * (2 * N * N + n * n)
        os.environ["RDXG_MEMORY_BUDGET"] = str(total - kept // 2)
        s = S.Solver(job, max_patches=64)
        assert s.recompute()
        assert int(s.debug("allocated_bytes")[0]) <= total - kept // 2
        s.close()
        # below even that: a clear error at creation
        os.environ["RDXG_MEMORY_BUDGET"] = str(1 << 20)
        with pytest.raises(S.SolverError, match="even with recomputed transforms"):
            S.Solver(job, max_patches=64)
    finally:
        del os.environ["RDXG_MEMORY_BUDGET"]
