"""Uneven batches: several handles of different geometries (OTF size, frames, modes, the fused
and the general path) solved in one CUDA graph with rdxg_solve_many, against each handle
solved alone (marked gpu)."""
import numpy as np
import pytest

from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu


def _handles():
    ws = [workload("plain64"), workload("production88", n_patches=2, frames=4), workload("large128", n_patches=1, frames=2)]
    out = []
    for w in ws:
        s = S.Solver(w.job, max_patches=w.patches.cutouts.shape[0])
        s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
        out.append(s)
    return ws, out


def test_many_equals_each_alone():
    # staged modes and per-patch convergence (FTOL as a relative metric change)
    st = S.SolveSettings(mode_start=5, mode_step=5, max_iterations=12, min_iterations=3, ftol=1e-6,
                         max_metrics=256)
    ws, hs = _handles()
    together = S.solve_many(hs, st)
    for w, s, got in zip(ws, hs, together):
        alone = s.run(st)
        np.testing.assert_array_equal(got["alpha"], alone["alpha"])
        for p in range(w.patches.cutouts.shape[0]):
            a, b = got["reports"][p], alone["reports"][p]
            assert (a.n_metrics, a.iterations, a.final_metric) == (b.n_metrics, b.iterations, b.final_metric)
            np.testing.assert_array_equal(got["metrics"][p, :a.n_metrics], alone["metrics"][p, :b.n_metrics])
        assert s.launch_count() > 0


def test_many_rejects_a_repeated_handle():
    ws, hs = _handles()
    st = S.fixed_iterations(ws[0].job.n_modes, 2, max_metrics=64)
    with pytest.raises(S.SolverError, match="twice"):
        S.solve_many([hs[0], hs[1], hs[0]], st)


def test_handles_of_different_sizes_keep_their_shared_memory():
    # the dynamic shared memory limit of a kernel is one process-wide attribute: a handle
    # created later with smaller needs (64 x 64, 8 images, 20 modes) must not lower it below
    # what an earlier one needs (64 x 64, 24 images, 60 modes: a larger tensor-core tile)
    from redux_gb300 import synth
    big_job = synth.make_job(64, 60, synth.LAYOUT_WB_NB(8), basis="kl", kl_last=121)
    big = synth.make_patches(big_job, 2, 15.0, np.random.default_rng(7))
    hb = S.Solver(big_job, max_patches=2)
    hb.set_patches(big.cutouts)
    w0 = workload("plain64")
    hs = S.Solver(w0.job, max_patches=1)
    hs.set_patches(w0.patches.cutouts, None, w0.patches.fixed_gamma)
    st = S.fixed_iterations(big_job.n_modes, 2, max_metrics=64)
    out = hb.run(st)
    assert all(r.n_metrics > 0 for r in out["reports"])
    L = hb.metric(big.alpha_true)
    assert np.all(np.isfinite(L))
