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


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_image_ft_and_gamma(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
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


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
@pytest.mark.parametrize("scale", [0.0, 0.5, 1.0])
def test_metric(cfg, scale):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    a = w.patches.alpha_true * scale
    L = s.metric(a)
    for p in range(a.shape[0]):
        Lo = _oracle(w, p).metric(a[p])
        assert abs(L[p] - Lo) <= TOL_METRIC * abs(Lo), (p, L[p], Lo)


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_otf(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    a = w.patches.alpha_true * 0.7
    s.gradient(a, "vogel")      # gradient evaluations keep the OTF in HBM
    otf = s.debug("otf")
    op = _oracle(w, 0)
    op.metric(a[0])
    ro = op.otf()
    rel = np.abs(otf[0] - ro).max() / np.abs(ro).max()
    assert rel < 1e-6, rel


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_gradient_vogel(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
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


# FP32 rounding (1e-7 in the metric) flips some of the line search's comparisons, and
# Brent's 10 % step tolerance turns each flip into a different accepted point, so FP32 and
# FP64 trajectories part after a few iterations and converge to different points of this
# non-convex metric (FP64 runs whose rounding differs part the same way).  Solves are
# therefore checked by what does not depend on the trajectory: the first evaluations, exact
# sequences in FP64, and -- below -- that the converged FP32 points are converged points of
# the FP64 metric (an FP64 continuation from them finds no more than it finds from FP64's own).


def test_solve_fixed_iterations(w0):
    job = w0.job
    s = _solver(w0)
    it = 20
    out = s.run(S.fixed_iterations(job.n_modes, it, max_metrics=64))
    ref = _oracle(w0).solve(oracle.default_cfg(max_iterations=it, n_modes=job.n_modes))
    rep = out["reports"][0]
    assert rep.iterations == it
    m = out["metrics"][0, :rep.n_metrics]
    # the first line searches see the same comparisons as the FP64 solver
    np.testing.assert_allclose(m[:3], ref["metrics"][:3], rtol=1e-5)
    assert np.all(np.diff(m) <= 0)                 # every iteration lowers the metric


# FP64 continuation of converged solves (FTOL 1e-6 on the relative metric change, 3
# consecutive, all modes at once): measured on the 225 production patches, the metric drop an
# FP64 handle still finds from the FP32 endpoints is 2.4e-5 median / 9.6e-5 max, from FP64's
# own endpoints 2.3e-5 / 1.1e-4 (the reference's stopping rule stops short of a minimum by
# about that much, in either precision).
TOL_CONTINUATION_MAX = 2e-4


def test_converged_fp32_points_are_fp64_converged():
    w = workload("production88", n_patches=8, frames=4)
    job = w.job
    M = job.n_modes
    conv = S.SolveSettings(mode_start=M, mode_step=M, max_iterations=2000, min_iterations=5, target_iterations=3,
                           ftol=1e-6, max_metrics=2100)
    s32 = _solver(w)
    a32 = s32.run(conv)["alpha"]
    s64 = _solver(w, "fp64")
    a64 = s64.run(conv)["alpha"]

    def drops(a):
        s64.set_start_alpha(a)
        reps = s64.run(conv)["reports"]
        return np.array([(r.initial_metric - r.final_metric) / r.initial_metric for r in reps])

    d32, d64 = drops(a32), drops(a64)
    print(f"\nFP64 continuation drop from FP32 endpoints: median {np.median(d32):.2e} max {d32.max():.2e}; "
          f"from FP64 endpoints: median {np.median(d64):.2e} max {d64.max():.2e}")
    assert np.all(d32 >= -1e-9) and np.all(d64 >= -1e-9)     # a continuation never goes up
    assert d32.max() <= TOL_CONTINUATION_MAX, d32
    assert np.median(d32) <= 2.0 * np.median(d64) + 1e-6, (np.median(d32), np.median(d64))


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_metric_with_stale_reference(cfg):
    """The line search evaluates the metric with the reference object of the last gradient
    point; the result must not depend on it beyond rounding."""
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    base = w.patches.alpha_true * 0.5
    g, _ = s.gradient(base, "vogel")
    d = -g / np.abs(g).max() * 1e-7
    tilt = np.zeros_like(base)
    tilt[..., 0] = 1e-7
    tilt[..., 1] = -1e-7
    for dd in (d, tilt):
        for t in (0.1, 1.0, 10.0):
            a = base + t * dd
            L = s.metric_with_reference(base, a)
            for p in range(a.shape[0]):
                Lo = _oracle(w, p).metric(a[p])
                assert abs(L[p] - Lo) <= TOL_METRIC * abs(Lo), (t, L[p], Lo)


def test_solve_fp64_same_evaluations(w0):
    job = w0.job
    s = _solver(w0, "fp64")
    it = 6
    out = s.run(S.fixed_iterations(job.n_modes, it, max_metrics=64))
    ref = _oracle(w0).solve(oracle.default_cfg(max_iterations=it, n_modes=job.n_modes))
    rep = out["reports"][0]
    assert rep.n_f_evals == ref["report"].n_f_evals
    np.testing.assert_allclose(out["metrics"][0, :rep.n_metrics], ref["metrics"], rtol=1e-9)


def _general_path_solver(w, precision="fp32"):
    import os
    os.environ["RDXG_NO_FUSED"] = "1"
    try:
        return _solver(w, precision)
    finally:
        del os.environ["RDXG_NO_FUSED"]


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_fused_and_general_paths_agree(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    sf = _solver(w)
    sg = _general_path_solver(w)
    a = w.patches.alpha_true * 0.6
    Lf, Lg = sf.metric(a), sg.metric(a)
    np.testing.assert_allclose(Lf, Lg, rtol=1e-6)
    gf, _ = sf.gradient(a, "vogel")
    gg, _ = sg.gradient(a, "vogel")
    assert np.linalg.norm(gf - gg) / np.linalg.norm(gg) < 1e-5


def test_staged_solve_with_reshifts(w0):
    """Two mode stages with one integer re-shift between them (SubImage::adjustShifts) against
    the FP64 oracle: the shift is decided by the coefficients after the first stage, whose
    line searches still agree with FP64."""
    job = w0.job
    kw = dict(max_iterations=3, min_iterations=3, ftol=1e-3)
    s = _solver(w0)
    out = s.run(S.SolveSettings(mode_start=5, mode_step=job.n_modes, max_metrics=64, **kw))
    op = _oracle(w0)
    ref = op.solve(oracle.Cfg(n_initial_modes=5, n_mode_increment=job.n_modes, target_iterations=3, fd_first=1,
                              eps=1e-10, brent_tol=0.1, **kw))
    rep = out["reports"][0]
    assert rep.iterations == ref["report"].iterations
    np.testing.assert_allclose(out["metrics"][0, :3], ref["metrics"][:3], rtol=1e-5)
    # images were re-cut between the stages on the GPU exactly as in the FP64 solver
    sg, so = s.debug("shifts")[0], op.shifts()[0]
    assert np.any(so != 0)
    np.testing.assert_array_equal(sg, so)


# restored object within 1e-4 relative of the FP64 oracle (relative to the image's peak)
TOL_RESTORE = 1e-4


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_restore(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    fc = w.job.otf_size / 2.0
    a = w.patches.alpha_true
    out = s.restore(a, fc)
    for p in range(a.shape[0]):
        ref = _oracle(w, p).restore(a[p], fc)
        for o in range(w.job.n_objects):
            err = np.abs(out[p, o] - ref[o]).max() / np.abs(ref[o]).max()
            assert err <= TOL_RESTORE, (p, o, err)


def test_restore_fp64_with_and_without_filter(w0):
    s = _solver(w0, precision="fp64")
    fc = w0.job.otf_size / 2.0
    a = w0.patches.alpha_true
    op = _oracle(w0)
    for nf in (False, True):
        out = s.restore(a, fc, no_filter=nf)
        ref = op.restore(a[0], fc, no_filter=nf)
        err = np.abs(out[0, 0] - ref[0]).max() / np.abs(ref[0]).max()
        assert err <= 1e-6, (nf, err)


# the general (unfused) FP32 path at N = 128 with 100 KL modes (the large-patch geometry, 2 frames)
def _w4():
    return workload("large128", n_patches=1, frames=2)


@pytest.mark.parametrize("scale", [0.0, 1.0])
def test_metric_n128_kl100(scale):
    w = _w4()
    s = _solver(w)
    a = w.patches.alpha_true * scale
    L = s.metric(a)
    Lo = _oracle(w).metric(a[0])
    assert abs(L[0] - Lo) <= TOL_METRIC * abs(Lo), (L[0], Lo)


def test_gradient_vogel_n128_kl100():
    w = _w4()
    s = _solver(w)
    a = w.patches.alpha_true * 0.5
    g, _ = s.gradient(a, "vogel")
    _, go = _oracle(w).gradient(a[0], method="vogel")
    rel = np.linalg.norm(g[0] - go) / np.linalg.norm(go)
    assert rel < TOL_GRAD, rel


def test_solve_n128_kl100_first_metrics():
    w = _w4()
    s = _solver(w)
    st = S.fixed_iterations(w.job.n_modes, 3, max_metrics=64)
    out = s.run(st)
    ref = _oracle(w).solve(oracle.Cfg(n_initial_modes=w.job.n_modes, n_mode_increment=w.job.n_modes,
                                      max_iterations=3, min_iterations=3, target_iterations=3, fd_first=1,
                                      ftol=0.0, eps=1e-10, brent_tol=0.1))
    n = min(3, out["reports"][0].n_metrics, len(ref["metrics"]))
    np.testing.assert_allclose(out["metrics"][0, :n], ref["metrics"][:n], rtol=1e-5)


def test_production_geometry_3x12():
    """The production geometry exactly (88 x 88, 36 KL modes, 3 channels x 12 frames), one patch
    of the production batch's generator: metric, Vogel and finite-difference gradients against
    the FP64 oracle, and the exact derivative against central differences of the oracle's
    metric on sampled entries."""
    w = workload("production88", n_patches=1, frames=12)
    job = w.job
    assert job.n_images == 36 and job.n_modes == 36
    s = _solver(w)
    op = _oracle(w)
    for scale in (0.0, 0.5, 1.0):
        a = w.patches.alpha_true * scale
        L = s.metric(a)[0]
        Lo = op.metric(a[0])
        assert abs(L - Lo) <= TOL_METRIC * abs(Lo), (scale, L, Lo)
    a = w.patches.alpha_true * 0.7
    g, _ = s.gradient(a, "vogel")
    _, go = op.gradient(a[0], "vogel")
    assert np.linalg.norm(g[0] - go) / np.linalg.norm(go) < TOL_GRAD
    gf, _ = s.gradient(a, "fd")
    _, gfo = op.gradient(a[0], "fd")
    assert np.linalg.norm(gf[0] - gfo) / np.linalg.norm(gfo) < 1e-4
    ge, _ = s.gradient(a, "exact")
    h = 1e-4 * job.wavelength
    rng = np.random.default_rng(7)
    for _ in range(6):
        j, m = int(rng.integers(job.n_images)), int(rng.integers(2, job.n_modes))
        ap = a[0].copy(); ap[j, m] += h
        am = a[0].copy(); am[j, m] -= h
        fd = (op.metric(ap) - op.metric(am)) / (2 * h)
        assert abs(ge[0, j, m] - fd) <= 1e-4 * max(abs(fd), 1e-3 * np.abs(ge[0]).max()), (j, m, ge[0, j, m], fd)


def test_fp64_n128_matches_oracle():
    """The FP64 form at N = 128 (its work tiles in global memory, a double tile exceeding a
    block's shared memory): metric, Vogel and finite-difference gradients against the FP64
    oracle, and a short solve with the oracle's evaluation sequence."""
    w = _w4()
    s = _solver(w, "fp64")
    op = _oracle(w)
    for scale in (0.0, 0.5, 1.0):
        a = w.patches.alpha_true * scale
        L = s.metric(a)[0]
        Lo = op.metric(a[0])
        assert abs(L - Lo) <= 1e-11 * abs(Lo), (scale, L, Lo)
    a = w.patches.alpha_true * 0.5
    g, _ = s.gradient(a, "vogel")
    _, go = op.gradient(a[0], "vogel")
    assert np.linalg.norm(g[0] - go) / np.linalg.norm(go) < 1e-10
    gf, _ = s.gradient(a, "fd")
    _, gfo = op.gradient(a[0], "fd")
    assert np.linalg.norm(gf[0] - gfo) / np.linalg.norm(gfo) < 1e-9
    it = 2
    out = s.run(S.fixed_iterations(w.job.n_modes, it, max_metrics=64))
    ref = op.solve(oracle.default_cfg(max_iterations=it, n_modes=w.job.n_modes))
    rep = out["reports"][0]
    assert rep.n_f_evals == ref["report"].n_f_evals
    np.testing.assert_allclose(out["metrics"][0, :rep.n_metrics], ref["metrics"], rtol=1e-9)
