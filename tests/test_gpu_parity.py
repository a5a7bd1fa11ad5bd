"""GPU solver vs the FP64 oracle through the C ABI (marked gpu)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu

# tolerances stated by the benchmark spec: metric and gradient within 1e-5 relative of FP64
TOL_METRIC = 1e-5
TOL_GRAD = 1e-5


def _oracle(w, p=0):
    op = oracle.OraclePatch(w.job)
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[p]
    op.set_images(w.patches.cutouts[p], None, fg)
    return op


def _solver(w, precision="fp32"):
    P = w.patches.cutouts.shape[0]
    s = S.Solver(w.job, max_patches=P, precision=precision)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return s


@pytest.mark.parametrize("cfg", [0, 2])
def test_image_ft_and_gamma(cfg):
    w = workload(0) if cfg == 0 else workload(2, n_patches=2, frames=4)
    s = _solver(w)
    D = s.debug("D")
    gam = s.debug("gamma")
    for p in range(D.shape[0]):
        op = _oracle(w, p)
        Do = op.D()
        rel = np.linalg.norm(D[p] - Do) / np.linalg.norm(Do)
        assert rel < 1e-6, rel
        np.testing.assert_allclose(gam[p], op.gamma(), rtol=1e-6)
        st = s.debug("stats")[p]
        m, sd, nz = op.stats()
        np.testing.assert_allclose(st[:, 0], m, rtol=1e-12)
        np.testing.assert_allclose(st[:, 1], sd, rtol=1e-9)
        np.testing.assert_allclose(st[:, 2], nz, rtol=1e-5)


@pytest.mark.parametrize("cfg", [0, 2])
@pytest.mark.parametrize("scale", [0.0, 0.5, 1.0])
def test_metric(cfg, scale):
    w = workload(0) if cfg == 0 else workload(2, n_patches=2, frames=4)
    s = _solver(w)
    a = w.patches.alpha_true * scale
    L = s.metric(a)
    for p in range(a.shape[0]):
        Lo = _oracle(w, p).metric(a[p])
        assert abs(L[p] - Lo) <= TOL_METRIC * abs(Lo), (p, L[p], Lo)


@pytest.mark.parametrize("cfg", [0, 2])
def test_otf(cfg):
    w = workload(0) if cfg == 0 else workload(2, n_patches=2, frames=4)
    s = _solver(w)
    a = w.patches.alpha_true * 0.7
    s.metric(a)
    otf = s.debug("otf")
    op = _oracle(w, 0)
    op.metric(a[0])
    ro = op.otf()
    rel = np.abs(otf[0] - ro).max() / np.abs(ro).max()
    assert rel < 1e-6, rel


@pytest.mark.parametrize("cfg", [0, 2])
def test_gradient_vogel(cfg):
    w = workload(0) if cfg == 0 else workload(2, n_patches=2, frames=4)
    s = _solver(w)
    a = w.patches.alpha_true * 0.5
    g, L = s.gradient(a, "vogel")
    for p in range(a.shape[0]):
        op = _oracle(w, p)
        Lo, go = op.gradient(a[p], "vogel")
        rel = np.linalg.norm(g[p] - go) / np.linalg.norm(go)
        assert rel < TOL_GRAD, rel
        assert abs(L[p] - Lo) <= TOL_METRIC * abs(Lo)


def test_gradient_exact_vs_central_fd(w0):
    s = _solver(w0)
    a = w0.patches.alpha_true * 0.5
    g, _ = s.gradient(a, "exact")
    op = _oracle(w0)
    h = 1e-4 * w0.job.wavelength
    I, M = w0.job.n_images, w0.job.n_modes
    gc = np.zeros((2, M))
    for j in range(2):
        for m in range(M):
            ap = a[0].copy(); ap[j, m] += h
            am = a[0].copy(); am[j, m] -= h
            gc[j, m] = (op.metric(ap) - op.metric(am)) / (2 * h)
    rel = np.linalg.norm(g[0, :2] - gc) / np.linalg.norm(gc)
    assert rel < 1e-4, rel


def test_gradient_fd(w0):
    s = _solver(w0)
    a = w0.patches.alpha_true * 0.5
    g, _ = s.gradient(a, "fd")
    _, go = _oracle(w0).gradient(a[0], "fd")
    rel = np.linalg.norm(g[0] - go) / np.linalg.norm(go)
    assert rel < 1e-4, rel


def test_fp64_mode_matches_oracle(w0):
    s = _solver(w0, "fp64")
    a = w0.patches.alpha_true * 0.5
    L = s.metric(a)[0]
    op = _oracle(w0)
    Lo = op.metric(a[0])
    assert abs(L - Lo) <= 1e-11 * abs(Lo)
    g, _ = s.gradient(a, "vogel")
    _, go = op.gradient(a[0], "vogel")
    assert np.linalg.norm(g[0] - go) / np.linalg.norm(go) < 1e-10


def test_solve_fixed_iterations(w0):
    job = w0.job
    s = _solver(w0)
    it = 20
    out = s.run(S.fixed_iterations(job.n_modes, it, max_metrics=64))
    ref = _oracle(w0).solve(oracle.default_cfg(max_iterations=it, n_modes=job.n_modes))
    rep = out["reports"][0]
    assert rep.iterations == it
    assert abs(rep.final_metric - ref["report"].final_metric) <= 1e-4 * ref["report"].final_metric
    da = (out["alpha"][0] - ref["alpha"]) / job.wavelength
    assert np.sqrt(np.mean(da ** 2)) < 1e-2


def test_solve_fp64_same_evaluations(w0):
    job = w0.job
    s = _solver(w0, "fp64")
    it = 6
    out = s.run(S.fixed_iterations(job.n_modes, it, max_metrics=64))
    ref = _oracle(w0).solve(oracle.default_cfg(max_iterations=it, n_modes=job.n_modes))
    rep = out["reports"][0]
    assert rep.n_f_evals == ref["report"].n_f_evals
    np.testing.assert_allclose(out["metrics"][0, :rep.n_metrics], ref["metrics"], rtol=1e-9)
