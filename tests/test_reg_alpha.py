"""REG_ALPHA: Solver::metric adds 0.5 sum alpha^2 w with Solver::regAlphaWeights
(solver.cpp:147-156, 804-811); Solver::gradient starts from alpha * w and assigns the data term
to the enabled modes, so alpha * w remains only for the modes not yet enabled
(solver.cpp:860-885).  The oracle on the CPU; the GPU against the oracle (marked gpu)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import jobsetup as js
from redux_gb300 import solver as S
from tests.conftest import workload


def _weights(job, reg_alpha=1.0):
    return js.reg_alpha_weights(np.sqrt(job.atm_var), job.n_images, job.patch_size, job.wavelength, reg_alpha)


def _oracle(w, weights=None, init=None):
    op = oracle.OraclePatch(w.job)
    op.set_reg_alpha(weights)
    op.set_initial_alpha(init)
    op.set_images(w.patches.cutouts[0], None, w.patches.fixed_gamma[0])
    return op


def test_weights_are_the_references(w0):
    job = w0.job
    W = _weights(job, 0.5)
    rms = np.sqrt(job.atm_var)
    assert W.shape == (job.n_images, job.n_modes)
    np.testing.assert_allclose(W[3], 0.5 / job.wavelength * job.n_images * job.patch_size ** 2 / rms ** 2)


def test_oracle_metric_and_gradient(w0):
    job = w0.job
    W = _weights(job, 1e3)
    a = w0.patches.alpha_true[0] * 0.5
    op0, op1 = _oracle(w0), _oracle(w0, W)
    L0, L1 = op0.metric(a), op1.metric(a)
    reg = 0.5 * np.sum(a * a * W)
    assert reg > 1e-6 * L0
    assert abs((L1 - L0) - reg) <= 1e-12 * L1
    en = np.zeros(job.n_modes, np.uint8)
    en[:5] = 1
    _, g0 = op0.gradient(a, "vogel", enabled=en)
    _, g1 = op1.gradient(a, "vogel", enabled=en)
    np.testing.assert_array_equal(g1[:, :5], g0[:, :5])           # enabled: the data term only
    np.testing.assert_allclose(g1[:, 5:], a[:, 5:] * W[:, 5:], rtol=1e-15)


@pytest.mark.gpu
def test_metric_gradient_and_staged_solve_against_the_oracle(w0):
    """Metric and gradient with REG_ALPHA at a point, then a staged solve (5 modes enabled
    first) from a warm start, so that the modes not yet enabled carry alpha * w into the
    free-parameter gradient on the device."""
    job = w0.job
    W = _weights(job, 1e3)
    a = w0.patches.alpha_true * 0.5
    s = S.Solver(job, max_patches=1)
    s.set_reg_alpha(W)
    s.set_patches(w0.patches.cutouts, None, w0.patches.fixed_gamma)
    op = _oracle(w0, W)
    Lo = op.metric(a[0])
    assert abs(s.metric(a)[0] - Lo) <= 1e-5 * abs(Lo)
    en = np.zeros(job.n_modes, np.uint8)
    en[:5] = 1
    g, _ = s.gradient(a, "vogel", enabled=en)
    _, go = op.gradient(a[0], "vogel", enabled=en)
    assert np.linalg.norm(g[0] - go) / np.linalg.norm(go) < 1e-5
    np.testing.assert_allclose(g[0][:, 5:], a[0][:, 5:] * W[:, 5:], rtol=1e-15)
    # staged solve from a warm start
    s.set_initial_alpha(a)
    kw = dict(max_iterations=3, min_iterations=3, ftol=1e-3)
    out = s.run(S.SolveSettings(mode_start=5, mode_step=job.n_modes, max_metrics=64, **kw))
    opw = _oracle(w0, W, init=a[0])
    ref = opw.solve(oracle.Cfg(n_initial_modes=5, n_mode_increment=job.n_modes, target_iterations=3, fd_first=1,
                               eps=1e-10, brent_tol=0.1, **kw))
    np.testing.assert_allclose(out["metrics"][0, :2], ref["metrics"][:2], rtol=1e-5)
    s.close()
