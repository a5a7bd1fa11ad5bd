"""Warm start (INIT_FILES): Solver::loadInit puts the initial coefficients in alpha_offset and
Solver::shiftAndInit(alpha_offset, true) re-cuts every image by the integer part of its tilt
before the images are set up (solver.cpp:412-413, 584-605; SubImage::adjustShifts,
subimage.cpp:444-480).  The oracle's shifts against a numpy statement of adjustShifts (CPU);
the GPU against the oracle (marked gpu)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S
from tests.conftest import workload


def _oracle(w, p=0, init=None):
    op = oracle.OraclePatch(w.job)
    op.set_initial_alpha(init)
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[p]
    op.set_images(w.patches.cutouts[p], None, fg)
    return op


def _np_shifts(job, alpha):
    """adjustShifts from zero shifts: -round(alphaToShift(alpha tilts)), limited to the cutout."""
    J = np.asarray(job.J_T_xy)
    ps, cs = job.patch_size, job.cutout_size
    margin = (cs - ps) // 2
    out = np.zeros((job.n_images, 2), np.int64)
    for j in range(job.n_images):
        ay, ax = alpha[j, job.tilt_y], alpha[j, job.tilt_x]
        want = (ax * J[1, 0] + ay * J[1, 1], ax * J[0, 0] + ay * J[0, 1])
        for d in range(2):
            nsh = -int(np.sign(want[d]) * np.floor(abs(want[d]) + 0.5))   # lround
            first, last = margin, margin + ps - 1
            if nsh + first < 0:
                nsh = -first
            if abs(nsh + last) >= cs:
                nsh = cs - last - 1
            out[j, d] = nsh
    return out


def test_oracle_shifts_follow_the_initial_tilts(w0):
    a0 = w0.patches.alpha_true[0]
    op = _oracle(w0, init=a0)
    ref = _np_shifts(w0.job, a0)
    assert np.any(ref != 0)
    np.testing.assert_array_equal(op.shifts()[0], ref)


def test_oracle_solve_starts_at_the_initial_coefficients(w0):
    a0 = w0.patches.alpha_true[0]
    warm = _oracle(w0, init=a0).solve(oracle.default_cfg(max_iterations=2, n_modes=w0.job.n_modes))
    cold = _oracle(w0).solve(oracle.default_cfg(max_iterations=2, n_modes=w0.job.n_modes))
    # the first metric is the metric at the initial coefficients on the re-cut images
    assert abs(warm["metrics"][0] - _oracle(w0, init=a0).metric(a0)) <= 1e-12 * warm["metrics"][0]
    assert warm["metrics"][0] < 0.5 * cold["metrics"][0]


@pytest.mark.gpu
def test_warm_start_against_the_oracle(w0):
    job = w0.job
    a0 = w0.patches.alpha_true
    s = S.Solver(job, max_patches=1)
    s.set_patches(w0.patches.cutouts, None, w0.patches.fixed_gamma)
    s.set_initial_alpha(a0)
    op = _oracle(w0, init=a0[0])
    np.testing.assert_array_equal(s.debug("shifts")[0], op.shifts()[0])
    Dg, Do = s.debug("D")[0], op.D()
    assert np.linalg.norm(Dg - Do) / np.linalg.norm(Do) < 1e-6
    out = s.run(S.fixed_iterations(job.n_modes, 3, max_metrics=16))
    ref = op.solve(oracle.default_cfg(max_iterations=3, n_modes=job.n_modes))
    np.testing.assert_allclose(out["metrics"][0, :2], ref["metrics"][:2], rtol=1e-5)
    # a second solve of the same batch starts from the same coefficients again
    out2 = s.run(S.fixed_iterations(job.n_modes, 3, max_metrics=16))
    np.testing.assert_array_equal(out2["metrics"], out["metrics"])
    # cleared: back to the cold start
    s.set_initial_alpha(None)
    cold = s.run(S.fixed_iterations(job.n_modes, 3, max_metrics=16))
    refc = _oracle(w0).solve(oracle.default_cfg(max_iterations=3, n_modes=job.n_modes))
    np.testing.assert_allclose(cold["metrics"][0, :2], refc["metrics"][:2], rtol=1e-5)
    s.close()
