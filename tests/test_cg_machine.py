"""The optimiser state machine (the code the device kernel runs) against the sequential
FP64 restatement of Solver::run / conjugate_rdx / bracket / brent in the oracle.

Driven on the host through rdxg_cg_minimize with the oracle's metric and gradient as
callbacks, the machine must request exactly the same evaluations and produce the same
metric history and coefficients, bit for bit."""
import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S


def _drive(w, settings):
    job = w.job
    op = oracle.OraclePatch(job)
    op.set_images(w.patches.cutouts[0], None, w.patches.fixed_gamma[0])
    M = job.n_modes
    st = {"off": np.zeros(job.n_images * M), "evals": 0}

    def f(x):
        st["evals"] += 1
        return op.metric(op.cons_reverse_add(x, st["off"]))

    def df(x, method, mc):
        a = op.cons_reverse_add(x, st["off"])
        en = np.zeros(M, np.uint8)
        en[:mc] = 1
        _, g = op.gradient(a, "vogel" if method == 2 else "fd", en)
        return op.cons_apply(g)

    def sh(x):
        a = op.cons_reverse_add(x, st["off"])
        op.shift(a)
        st["off"] = a

    n_tot = job.n_images * job.patch_size ** 2
    out = S.cg_minimize(job.nullspace.n_free, M, settings, 1.0 / n_tot ** 2, f, df, sh)
    return out, op.cons_reverse_add(out["x"], st["off"]), op


def _reference(w, settings):
    op = oracle.OraclePatch(w.job)
    op.set_images(w.patches.cutouts[0], None, w.patches.fixed_gamma[0])
    cfg = oracle.Cfg(n_initial_modes=settings.mode_start, n_mode_increment=settings.mode_step,
                     max_iterations=settings.max_iterations, min_iterations=settings.min_iterations,
                     target_iterations=settings.target_iterations, fd_first=int(settings.fd_first),
                     ftol=settings.ftol, eps=settings.eps, brent_tol=0.1)
    return op.solve(cfg), op


@pytest.mark.parametrize("settings", [
    S.fixed_iterations(20, 6, max_metrics=64),
    S.SolveSettings(mode_start=5, mode_step=5, max_iterations=10, min_iterations=3, ftol=1e-3, max_metrics=128),
], ids=["fixed", "staged"])
def test_machine_matches_sequential_solver(w0, settings):
    out, alpha, op = _drive(w0, settings)
    ref, opr = _reference(w0, settings)
    assert out["report"].n_f_evals == ref["report"].n_f_evals
    assert out["report"].n_df_evals == ref["report"].n_df_evals
    assert out["report"].iterations == ref["report"].iterations
    np.testing.assert_array_equal(out["metrics"], ref["metrics"])
    np.testing.assert_array_equal(alpha, ref["alpha"].ravel())
    # the staged run re-shifted images between stages exactly as the sequential solver
    s1, t1 = op.shifts()
    s2, t2 = opr.shifts()
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(t1, t2)


def test_quadratic_converges():
    """On a convex quadratic the minimiser reaches the minimum.  The reference's first trial
    step is 1e-21 times the search direction (conjugate_gradient.cpp:203), tuned to MOMFBD's
    units (coefficients ~1e-7, metrics ~1e9, gradients ~1e16), so the test uses that scale."""
    n = 12
    rng = np.random.default_rng(3)
    A = rng.standard_normal((n, n))
    H = A @ A.T + n * np.eye(n)
    b = rng.standard_normal(n)
    sig, s = 1e-7, 1e9
    xs = np.linalg.solve(H, b) * sig
    f = lambda x: s * float(0.5 * (x / sig) @ H @ (x / sig) - b @ (x / sig)) + 1e10
    df = lambda x, m, mc: s * (H @ (x / sig) - b) / sig
    out = S.cg_minimize(n, 1, S.SolveSettings(mode_start=1, mode_step=1, max_iterations=40, min_iterations=40,
                                               ftol=0.0, fd_first=False, max_metrics=128), 1.0, f, df)
    assert np.abs(out["x"] - xs).max() < 1e-4 * np.abs(xs).max()
