"""The solver kernel's two forms (rdxg_launch_shape.solver_form): staged, with the patch's
optimiser vectors, object metric sums, object tables and null-space map copied into shared
memory as the kernel starts, and the global-memory form.  They perform the same arithmetic in
the same order, so every solve must give the same bits either way: coefficients, metric
histories, evaluation counts -- on the fused 88 x 88 path with staged modes and re-shifts, with
REG_ALPHA, on a ragged batch, on the general 128 x 128 path and in FP64 (marked gpu)."""
import numpy as np
import pytest

from redux_gb300 import solver as S, synth
from tests.conftest import workload

pytestmark = pytest.mark.gpu

STAGED = S.SolveSettings(mode_start=5, mode_step=5, max_iterations=4, min_iterations=2, ftol=1e-6, max_metrics=512)


def _solve(make, form):
    s, settings = make()
    s.set_launch_shape(solver_form=form)
    assert s.launch_shape()["solver_form"] == form
    out = s.run(settings)
    s.close()
    return out


def _fused88():
    w = workload("production88", n_patches=2, frames=4)
    s = S.Solver(w.job, max_patches=2)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return s, STAGED


def _reg_alpha():
    w = workload("production88", n_patches=2, frames=4)
    s = S.Solver(w.job, max_patches=2)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    rng = np.random.default_rng(5)
    s.set_reg_alpha(rng.uniform(0.5, 2.0, (w.job.n_images, w.job.n_modes)) * 1e-3)
    return s, S.fixed_iterations(w.job.n_modes, 4, max_metrics=64)


def _ragged():
    N, F_max, M_max = 88, 5, 40
    shapes, assign = [(3, 36), (5, 40), (2, 38)], [0, 1, 2, 1]
    kl = synth.UNEVEN_KL_LAST
    big = synth.make_job(N, M_max, synth.LAYOUT_WB_NB(F_max), basis="kl", kl_last=kl)
    jobs = [synth.make_job(N, M, synth.LAYOUT_WB_NB(F), basis="kl", kl_last=kl) for F, M in shapes]
    rng = np.random.default_rng(21)
    packed = np.zeros((len(assign), big.n_images, big.cutout_size, big.cutout_size), np.float32)
    for p, k in enumerate(assign):
        packed[p, :jobs[k].n_images] = synth.make_patches(jobs[k], 1, 12.0, rng).cutouts[0]
    s = S.Solver(big, max_patches=len(assign))
    s.set_patch_shapes([(F, M, j.nullspace) for (F, M), j in zip(shapes, jobs)], assign)
    s.set_patches(packed)
    return s, STAGED


def _general128():
    w = workload("large128", n_patches=1, frames=2)
    s = S.Solver(w.job, max_patches=1)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return s, S.fixed_iterations(w.job.n_modes, 3, max_metrics=32)


def _fp64():
    w = workload("plain64")
    s = S.Solver(w.job, max_patches=w.patches.cutouts.shape[0], precision="fp64")
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return s, STAGED


CASES = {"fused88": _fused88, "reg_alpha": _reg_alpha, "ragged": _ragged, "general128": _general128,
         "fp64": _fp64}


@pytest.mark.parametrize("case", sorted(CASES))
def test_staged_and_global_forms_give_identical_solves(case):
    make = CASES[case]
    a = _solve(make, 1)
    b = _solve(make, 2)
    np.testing.assert_array_equal(a["alpha"], b["alpha"])
    np.testing.assert_array_equal(a["metrics"], b["metrics"])
    for ra, rb in zip(a["reports"], b["reports"]):
        assert (ra.iterations, ra.status, ra.n_f_evals, ra.n_df_evals, ra.n_metrics) == \
            (rb.iterations, rb.status, rb.n_f_evals, rb.n_df_evals, rb.n_metrics)
        assert ra.final_metric == rb.final_metric


def test_solver_form_rejects_unknown_values():
    w = workload("plain64")
    s = S.Solver(w.job, max_patches=1)
    with pytest.raises(S.SolverError, match="solver_form"):
        s.set_launch_shape(solver_form=3)
    s.close()
