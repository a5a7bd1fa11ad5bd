"""The conjugate-gradient iteration and line search pinned to the reference's own compiled code.

oracle/_ref/libref_cg.so holds redux's conjugate_rdx minimiser and its bracket and brent
(src/lib/util/gsl/conjugate_gradient.cpp, src/lib/math/helpers.cpp), compiled from the
reference's sources (`make -C oracle ref`), under the stage loop of Solver::run.  Three
implementations are driven with the same callbacks and must agree bit for bit -- the metric
history, every count of the report and the final point:
  * the reference's compiled minimiser (oracle.ref_cg_minimize),
  * the oracle's sequential restatement (oracle.cg_minimize, the code every GPU parity test
    compares against),
  * the product's optimiser state machine, the code the solver kernel runs, driven on the host
    (rdxg_cg_minimize).
The callbacks are analytic functions at MOMFBD's scale, the oracle's FP64 metric and gradient
of a patch, and the same with failures injected on the host (a non-finite metric, a zero or
non-finite gradient) to exercise Solver::run's failure handling (solver.cpp:470-499) and
conjugate_rdx_iterate's no-progress exits (conjugate_gradient.cpp:158-161, 192-195)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S

if not oracle.ref_available() and not oracle.build_ref():
    pytest.skip("the reference's minimiser is not built (its sources are not present)", allow_module_level=True)


def _settings(cfg: "oracle.Cfg") -> S.SolveSettings:
    return S.SolveSettings(mode_start=cfg.n_initial_modes, mode_step=cfg.n_mode_increment,
                           max_iterations=cfg.max_iterations, min_iterations=cfg.min_iterations,
                           target_iterations=cfg.target_iterations, fd_first=bool(cfg.fd_first), ftol=cfg.ftol,
                           eps=cfg.eps, max_metrics=100000)


def _cfg(n_initial, step, max_it, min_it=None, ftol=0.0, fd_first=1, target=3):
    return oracle.Cfg(n_initial_modes=n_initial, n_mode_increment=step, max_iterations=max_it,
                      min_iterations=max_it if min_it is None else min_it, target_iterations=target,
                      fd_first=fd_first, ftol=ftol, eps=1e-10, brent_tol=0.1)


def _run_all(n_free, n_modes, cfg, grad_scale, make_problem):
    """make_problem() -> (f, df, shift, log): fresh callbacks for each implementation."""
    outs = {}
    for name in ("reference", "oracle", "machine"):
        f, df, sh, log = make_problem()
        if name == "reference":
            o = oracle.ref_cg_minimize(n_free, n_modes, cfg, grad_scale, f, df, sh)
        elif name == "oracle":
            o = oracle.cg_minimize(n_free, n_modes, cfg, grad_scale, f, df, sh)
        else:
            o = S.cg_minimize(n_free, n_modes, _settings(cfg), grad_scale, f, df, sh)
            o["metrics"] = o["metrics"][:o["report"].n_metrics]
        o["log"] = log
        outs[name] = o
    return outs


def _assert_same(outs):
    ref = outs["reference"]
    r = ref["report"]
    for name in ("oracle", "machine"):
        o = outs[name]
        q = o["report"]
        for fld in ("iterations", "status", "n_f_evals", "n_df_evals", "fail_count", "n_metrics"):
            assert getattr(q, fld) == getattr(r, fld), (name, fld, getattr(q, fld), getattr(r, fld))
        np.testing.assert_array_equal(o["metrics"], ref["metrics"], err_msg=name)
        np.testing.assert_array_equal(o["x"], ref["x"], err_msg=name)
        for k in ("initial_metric", "final_metric"):
            a, b = getattr(q, k), getattr(r, k)
            assert (a == b) or (np.isnan(a) and np.isnan(b)), (name, k, a, b)
        assert o["log"] == ref["log"], name        # the same sequence of requests


# ---- analytic problems at the reference's scale (coefficients ~1e-7, metrics ~1e9) ----
SIG, SCALE = 1e-7, 1e9


def _quadratic(n, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((n, n))
    H = A @ A.T + n * np.eye(n)
    b = rng.standard_normal(n)
    return H, b


def _problem_factory(n, seed, kind="quadratic", fail=None):
    H, b = _quadratic(n, seed)

    def make():
        log = []
        st = {"nf": 0, "ndf": 0, "off": np.zeros(n)}

        def value(x):
            y = (x + st["off"]) / SIG
            v = 0.5 * y @ H @ y - b @ y
            if kind == "nonconvex":
                v += 3.0 * np.sum(np.cos(1.7 * y))
            return SCALE * float(v) + 1e10

        def grad(x):
            y = (x + st["off"]) / SIG
            g = H @ y - b
            if kind == "nonconvex":
                g = g - 3.0 * 1.7 * np.sin(1.7 * y)
            return SCALE * g / SIG

        def f(x):
            st["nf"] += 1
            log.append(("f",))
            v = value(x)
            if fail == "nan_metric" and st["nf"] > 30:
                return float("nan")
            return v

        def df(x, method, mc):
            st["ndf"] += 1
            log.append(("df", method, mc))
            g = grad(x)
            g[mc:] = 0.0                      # modes not yet enabled (one parameter per mode here)
            if fail == "zero_gradient" and st["ndf"] >= 3:
                return np.zeros(n)
            if fail == "inf_gradient" and st["ndf"] >= 3:
                g[0] = np.inf
            if fail == "nan_gradient" and st["ndf"] >= 2:
                g[1] = np.nan
            return g

        def shift(x):
            log.append(("shift",))
            st["off"] = st["off"] + x          # alpha_offset = alpha

        return f, df, shift, log

    return make


@pytest.mark.parametrize("kind", ["quadratic", "nonconvex"])
@pytest.mark.parametrize("staged", [False, True], ids=["all_modes", "staged"])
def test_analytic_problems(kind, staged):
    n = 16
    cfg = _cfg(4, 4, 12, min_it=3, ftol=1e-9) if staged else _cfg(n, n, 25)
    outs = _run_all(n, n, cfg, 1.0, _problem_factory(n, 7, kind))
    _assert_same(outs)
    assert outs["reference"]["report"].iterations >= (12 if not staged else 4)


def test_nan_metric_gives_up_after_more_than_three_failures():
    """Every metric after the 30th is NaN: each mode stage ends at its first iteration with a
    failure (non-finite metric) until the fourth, after which Solver::run gives up (status 1)."""
    n = 20
    cfg = _cfg(2, 2, 10, min_it=2, ftol=1e-12)
    outs = _run_all(n, n, cfg, 1.0, _problem_factory(n, 11, fail="nan_metric"))
    _assert_same(outs)
    r = outs["reference"]["report"]
    assert r.status == 1 and r.fail_count == 4, (r.status, r.fail_count)


@pytest.mark.parametrize("fail", ["zero_gradient", "inf_gradient", "nan_gradient"])
def test_gradient_failures(fail):
    """A zero gradient ends the iteration with GSL_ENOPROG (pnorm = 0); a non-finite one makes
    the gradient norm non-finite.  Either counts as a failure and ends the stage."""
    n = 20
    cfg = _cfg(2, 2, 10, min_it=2, ftol=1e-12)
    outs = _run_all(n, n, cfg, 1.0, _problem_factory(n, 5, fail=fail))
    _assert_same(outs)
    assert outs["reference"]["report"].fail_count >= 1


# ---- the oracle's FP64 metric and gradient of a patch ----
def _patch_factory(w):
    job = w.job
    M = job.n_modes

    def make():
        op = oracle.OraclePatch(job)
        op.set_images(w.patches.cutouts[0], None, w.patches.fixed_gamma[0])
        st = {"off": np.zeros(job.n_images * M)}
        log = []

        def f(x):
            log.append(("f",))
            return op.metric(op.cons_reverse_add(x, st["off"]))

        def df(x, method, mc):
            log.append(("df", method, mc))
            a = op.cons_reverse_add(x, st["off"])
            en = np.zeros(M, np.uint8)
            en[:mc] = 1
            _, g = op.gradient(a, "vogel" if method == 2 else "fd", en)
            return op.cons_apply(g)

        def sh(x):
            log.append(("shift",))
            a = op.cons_reverse_add(x, st["off"])
            op.shift(a)
            st["off"] = a

        return f, df, sh, log

    return make


@pytest.mark.parametrize("staged", [False, True], ids=["fixed", "staged"])
def test_oracle_patch(w0, staged):
    job = w0.job
    cfg = _cfg(5, 5, 8, min_it=3, ftol=1e-3) if staged else _cfg(job.n_modes, job.n_modes, 5)
    n_tot = job.n_images * job.patch_size ** 2
    outs = _run_all(job.nullspace.n_free, job.n_modes, cfg, 1.0 / n_tot ** 2, _patch_factory(w0))
    _assert_same(outs)
    # and the oracle's own patch solver (orc_solve) takes the same path
    op = oracle.OraclePatch(job)
    op.set_images(w0.patches.cutouts[0], None, w0.patches.fixed_gamma[0])
    ref = op.solve(cfg)
    np.testing.assert_array_equal(ref["metrics"], outs["reference"]["metrics"])
    assert ref["report"].n_f_evals == outs["reference"]["report"].n_f_evals
