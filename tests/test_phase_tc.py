"""Mode expansion on the tensor cores (tcgen05, BF16 parts with FP32 accumulation) through the
C ABI: rdxg_set_phase_mode 3 (6xBF16, the default), 2 (3xBF16) and 0 (CUDA cores, FP32),
against each other and against the FP64 oracle (marked gpu)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu

TOL_METRIC = 1e-5
TOL_GRAD = 1e-5
# phases against the FP32 CUDA-core expansion, relative to the largest |phi| of the batch:
# 6xBF16 drops only products below 2^-24 (measured 2.3e-7 ... 2.8e-7), 3xBF16 drops
# x1*y1 ~ 2^-18 per term (measured 6.2e-6 ... 6.3e-6)
TOL_PHASE = {3: 1e-6, 2: 2e-5}


def _w(cfg):
    return workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)


def _solver(w):
    P = w.patches.cutouts.shape[0]
    s = S.Solver(w.job, max_patches=P, precision="fp32")
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return s


def _oracle(w, p=0):
    op = oracle.OraclePatch(w.job)
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[p]
    op.set_images(w.patches.cutouts[p], None, fg)
    return op


def test_default_is_6xbf16():
    s = _solver(_w("plain64"))
    assert s.phase_mode() == 3


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_phases_against_cuda_cores(cfg):
    w = _w(cfg)
    s = _solver(w)
    a = w.patches.alpha_true
    ph = {}
    for mode in (0, 2, 3):
        s.set_phase_mode(mode)
        assert s.phase_mode() == mode
        s.metric(a)
        ph[mode] = s.debug("phases").astype(np.float64)
    scale = np.abs(ph[0]).max()
    for mode in (2, 3):
        err = np.abs(ph[mode] - ph[0]).max() / scale
        assert err <= TOL_PHASE[mode], (mode, err)


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
@pytest.mark.parametrize("mode", [0, 2, 3])
def test_metric_each_mode(cfg, mode):
    w = _w(cfg)
    s = _solver(w)
    s.set_phase_mode(mode)
    for scale in (0.5, 1.0):
        a = w.patches.alpha_true * scale
        L = s.metric(a)
        for p in range(a.shape[0]):
            Lo = _oracle(w, p).metric(a[p])
            assert abs(L[p] - Lo) <= TOL_METRIC * abs(Lo), (mode, scale, p, L[p], Lo)


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_gradient_6xbf16(cfg):
    w = _w(cfg)
    s = _solver(w)
    s.set_phase_mode(3)
    a = w.patches.alpha_true * 0.7
    g, _ = s.gradient(a, "vogel")
    _, go = _oracle(w).gradient(a[0], method="vogel")
    rel = np.linalg.norm(g[0] - go) / np.linalg.norm(go)
    assert rel < TOL_GRAD, rel


def test_gradient_3xbf16_error_is_bounded():
    # the 3xBF16 split misses the 1e-5 gradient tolerance at 64 x 64 with Zernike phases of
    # up to 65 rad (measured 2.5e-5); it stays within 5e-5
    w = _w("plain64")
    s = _solver(w)
    s.set_phase_mode(2)
    a = w.patches.alpha_true * 0.7
    g, _ = s.gradient(a, "vogel")
    _, go = _oracle(w).gradient(a[0], method="vogel")
    rel = np.linalg.norm(g[0] - go) / np.linalg.norm(go)
    assert rel < 5e-5, rel


def test_solve_first_metrics_6xbf16():
    w = _w("plain64")
    s = _solver(w)
    s.set_phase_mode(3)
    st = S.fixed_iterations(w.job.n_modes, 3, max_metrics=64)
    out = s.run(st)
    ref = _oracle(w).solve(oracle.Cfg(n_initial_modes=w.job.n_modes, n_mode_increment=w.job.n_modes,
                                      max_iterations=3, min_iterations=3, target_iterations=3, fd_first=1,
                                      ftol=0.0, eps=1e-10, brent_tol=0.1))
    n = min(3, out["reports"][0].n_metrics, len(ref["metrics"]))
    np.testing.assert_allclose(out["metrics"][0, :n], ref["metrics"][:n], rtol=1e-5)


def test_mode_errors():
    w = _w("plain64")
    s = _solver(w)
    with pytest.raises(S.SolverError):
        s.set_phase_mode(1)
    assert s.phase_mode() == 3
    s64 = S.Solver(w.job, max_patches=1, precision="fp64")
    s64.set_phase_mode(0)
    with pytest.raises(S.SolverError, match="general path"):
        s64.set_phase_mode(3)
    assert s64.phase_mode() == 0


# phases on the pupil support against FP64 phi_fixed + sum alpha Z (numpy), in rad: the
# 6xBF16 split is at the level of FP32 rounding, 3xBF16 keeps ~2^-18 of each product
TOL_PHASE_RAD = {0: 3e-5, 3: 3e-5, 2: 5e-4}


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_phases_against_fp64(cfg):
    w = _w(cfg)
    job = w.job
    s = _solver(w)
    a = w.patches.alpha_true
    n2 = job.pupil_pixels ** 2
    Z = job.modes.reshape(job.n_modes, n2)
    pf = job.phi_fixed.reshape(-1, n2)[job.img_channel]              # [I][n2]
    ref = np.einsum("pim,mq->piq", a, Z) + pf[None]
    sup = np.asarray(job.pupil).ravel() > 0
    errs = {}
    for mode in (0, 2, 3):
        s.set_phase_mode(mode)
        s.metric(a)
        ph = s.debug("phases").astype(np.float64).reshape(ref.shape)
        errs[mode] = np.abs(ph - ref)[..., sup].max()
    print(f"phase error vs FP64 on the pupil (rad): {errs}")
    for mode, e in errs.items():
        assert e <= TOL_PHASE_RAD[mode], (mode, e)
    assert errs[3] <= errs[2]


@pytest.mark.parametrize("word, what", [(1, "mode tile copy"), (2, "products")])
def test_status_word_reported_once(word, what):
    """A bounded wait of the tensor-core kernel that gives up leaves a status word; the host
    reports it as an error on the next call and clears it.  The word is written from the host
    (no wait is made to run out on the GPU)."""
    w = _w("plain64")
    s = _solver(w)
    a = w.patches.alpha_true * 0.5
    ok = s.metric(a)
    s.debug_set_tc_status(word)
    with pytest.raises(S.SolverError, match=what):
        s.metric(a)
    np.testing.assert_allclose(s.metric(a), ok, rtol=1e-6)    # cleared, the handle still works


# the general path (OTF size 128, 100 KL modes): the same tensor-core expansion ahead of the
# transform kernel
def _w128():
    return workload("large128", n_patches=1, frames=2)


def test_general_path_default_is_6xbf16():
    s = _solver(_w128())
    assert s.phase_mode() == 3


def test_general_path_phases_against_fp64():
    w = _w128()
    job = w.job
    s = _solver(w)
    a = w.patches.alpha_true
    n2 = job.pupil_pixels ** 2
    Z = job.modes.reshape(job.n_modes, n2)
    pf = job.phi_fixed.reshape(-1, n2)[job.img_channel]
    ref = np.einsum("pim,mq->piq", a, Z) + pf[None]
    sup = np.asarray(job.pupil).ravel() > 0
    errs = {}
    for mode in (2, 3):
        s.set_phase_mode(mode)
        s.metric(a)
        ph = s.debug("phases").astype(np.float64).reshape(ref.shape)
        errs[mode] = np.abs(ph - ref)[..., sup].max()
    print(f"general path (128, 100 KL): phase error vs FP64 on the pupil (rad): {errs}")
    assert errs[3] <= TOL_PHASE_RAD[3] and errs[2] <= TOL_PHASE_RAD[2], errs


@pytest.mark.parametrize("mode", [0, 2, 3])
def test_general_path_metric_and_gradient_each_mode(mode):
    w = _w128()
    s = _solver(w)
    s.set_phase_mode(mode)
    assert s.phase_mode() == mode
    a = w.patches.alpha_true * 0.5
    op = _oracle(w)
    L = s.metric(a)[0]
    Lo = op.metric(a[0])
    assert abs(L - Lo) <= TOL_METRIC * abs(Lo), (mode, L, Lo)
    g, _ = s.gradient(a, "vogel")
    _, go = op.gradient(a[0], method="vogel")
    rel = np.linalg.norm(g[0] - go) / np.linalg.norm(go)
    assert rel < (5e-5 if mode == 2 else TOL_GRAD), (mode, rel)


def test_general_path_solve_6xbf16():
    w = _w128()
    s = _solver(w)
    st = S.fixed_iterations(w.job.n_modes, 3, max_metrics=64)
    out = s.run(st)
    ref = _oracle(w).solve(oracle.Cfg(n_initial_modes=w.job.n_modes, n_mode_increment=w.job.n_modes,
                                      max_iterations=3, min_iterations=3, target_iterations=3, fd_first=1,
                                      ftol=0.0, eps=1e-10, brent_tol=0.1))
    n = min(3, out["reports"][0].n_metrics, len(ref["metrics"]))
    np.testing.assert_allclose(out["metrics"][0, :n], ref["metrics"][:n], rtol=1e-5)
