"""Adjoint check (88x88, 3 channels x 8 frames, 36 KL modes, FP32 forward): the device
gradient at 20 seeded random points, against the reference's analytic (Vogel) gradient in
the FP64 oracle, and the exact derivative against central finite differences of the FP64
oracle metric (h = 1e-4 rad).  Prints the relative-error distributions (pytest -s), with the
per-image transforms kept from the evaluation and recomputed by the gradient kernels
(rdxg_set_recompute)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu

N_POINTS = 20
TOL_GRAD = 1e-5        # gradient within 1e-5 relative (norm) of the FP64 reference gradient
TOL_FD = 1e-4          # exact derivative against FP64 central differences (sampled entries)


@pytest.mark.parametrize("recompute", [False, True], ids=["kept", "recomputed"])
def test_adjoint_check_88x88_3x8_36kl(recompute):
    w = workload("adjoint88", n_patches=1)
    job = w.job
    I, M = job.n_images, job.n_modes
    s = S.Solver(job, max_patches=1)
    s.set_recompute(recompute)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    op = oracle.OraclePatch(job)
    op.set_images(w.patches.cutouts[0], None, None)
    rng = np.random.default_rng(20261203 + 1)
    a0 = w.patches.alpha_true[0]
    scale = np.abs(a0).max()
    h = 1e-4 * job.wavelength
    rel_vogel, rel_fd = [], []
    for k in range(N_POINTS):
        a = a0 + 0.3 * scale * rng.standard_normal(a0.shape)
        g_dev, _ = s.gradient(a[None], "vogel")
        _, g_ref = op.gradient(a, method="vogel")
        rel_vogel.append(np.linalg.norm(g_dev[0] - g_ref) / np.linalg.norm(g_ref))
        ge, _ = s.gradient(a[None], "exact")
        idx = [(int(rng.integers(I)), int(rng.integers(M))) for _ in range(4)]
        for j, m in idx:
            ap = a.copy(); ap[j, m] += h
            am = a.copy(); am[j, m] -= h
            fd = (op.metric(ap) - op.metric(am)) / (2 * h)
            rel_fd.append(abs(ge[0, j, m] - fd) / max(abs(fd), 1e-3 * np.abs(ge[0]).max()))
    rv, rf = np.array(rel_vogel), np.array(rel_fd)
    print(f"\n[transforms {'recomputed' if recompute else 'kept'}]")
    print(f"Vogel vs FP64 oracle (norm, {N_POINTS} points): median {np.median(rv):.2e} max {rv.max():.2e}")
    print(f"exact vs FP64 central differences ({rf.size} entries): median {np.median(rf):.2e} "
          f"p90 {np.percentile(rf, 90):.2e} max {rf.max():.2e}")
    assert rv.max() <= TOL_GRAD, rv.max()
    assert rf.max() <= TOL_FD, rf.max()
