"""Ragged batches (rdxg_set_patch_shapes): patches of one OTF size whose frames per channel and
mode counts differ, in one handle.  redux solves each such patch in the job of its own
geometry (momfbdjob.cpp:576-591); here every patch of a ragged handle must give exactly what a
handle of its own geometry gives for it -- metrics, gradients, the solve's metric history and
coefficients, bit for bit -- on the fused 88 x 88 path and the general 128 x 128 path (marked
gpu).  The modes are the first n_modes of one Karhunen-Loeve expansion (as in the uneven
benchmark), so every geometry's modes are a prefix of the handle's."""
import numpy as np
import pytest

from redux_gb300 import solver as S, synth

pytestmark = pytest.mark.gpu

KL_LAST = synth.UNEVEN_KL_LAST


def _case(N, F_max, M_max, shapes, assign, seed):
    """The handle's job (F_max frames, M_max modes), one job per shape, and per patch its
    own-geometry cutouts and the same images packed into the handle's slots."""
    layout = synth.LAYOUT_WB_NB
    big = synth.make_job(N, M_max, layout(F_max), basis="kl", kl_last=KL_LAST)
    jobs = [synth.make_job(N, M, layout(F), basis="kl", kl_last=KL_LAST) for F, M in shapes]
    rng = np.random.default_rng(seed)
    own, packed = [], np.zeros((len(assign), big.n_images, big.cutout_size, big.cutout_size), np.float32)
    for p, k in enumerate(assign):
        pt = synth.make_patches(jobs[k], 1, 12.0, rng)
        own.append(pt)
        packed[p, :jobs[k].n_images] = pt.cutouts[0]
    return big, jobs, own, packed


def _ragged(big, jobs, shapes, assign, packed, **kw):
    s = S.Solver(big, max_patches=len(assign), **kw)
    s.set_patch_shapes([(F, M, j.nullspace) for (F, M), j in zip(shapes, jobs)], assign)
    s.set_patches(packed)
    return s


def _embed(a, big, job):
    """[I_p][M_p] coefficients of a patch -> the handle's [I][M] layout."""
    out = np.zeros((big.n_images, big.n_modes))
    out[:job.n_images, :job.n_modes] = a
    return out


CASES = {
    # fused half-plane path, 3 channels x up to 5 frames, up to 40 KL modes
    "fused88": dict(N=88, F_max=5, M_max=40, shapes=[(3, 36), (5, 40), (2, 38), (5, 36)],
                    assign=[0, 1, 2, 3, 1, 0], seed=11),
    # general path with the tensor-core mode expansion, 3 channels x up to 2 frames
    "general128": dict(N=128, F_max=2, M_max=24, shapes=[(1, 20), (2, 24)], assign=[1, 0, 1], seed=12),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_ragged_patches_equal_their_own_geometry(case):
    c = CASES[case]
    big, jobs, own, packed = _case(**c)
    shapes, assign = c["shapes"], c["assign"]
    rs = _ragged(big, jobs, shapes, assign, packed)
    # single evaluations at each patch's true coefficients
    a_all = np.stack([_embed(own[p].alpha_true[0], big, jobs[k]) for p, k in enumerate(assign)])
    L = rs.metric(a_all)
    g, _ = rs.gradient(a_all, "vogel")
    # a staged solve (re-shifts between mode stages, per-patch stops)
    st = S.SolveSettings(mode_start=5, mode_step=5, max_iterations=4, min_iterations=2, ftol=1e-6, max_metrics=512)
    out = rs.run(st)
    fc = c["N"] / 2.0
    obj = rs.restore(out["alpha"], fc)
    for p, k in enumerate(assign):
        job = jobs[k]
        s1 = S.Solver(job, max_patches=1)
        s1.set_patches(own[p].cutouts)
        L1 = s1.metric(own[p].alpha_true)
        g1, _ = s1.gradient(own[p].alpha_true, "vogel")
        o1 = s1.run(st)
        obj1 = s1.restore(o1["alpha"], fc)
        s1.close()
        I, M = job.n_images, job.n_modes
        np.testing.assert_array_equal(L[p], L1[0], err_msg=f"patch {p} metric")
        np.testing.assert_array_equal(g[p][:I, :M], g1[0], err_msg=f"patch {p} gradient")
        r, r1 = out["reports"][p], o1["reports"][0]
        assert (r.iterations, r.n_f_evals, r.n_df_evals, r.n_metrics) == \
            (r1.iterations, r1.n_f_evals, r1.n_df_evals, r1.n_metrics), p
        np.testing.assert_array_equal(out["metrics"][p, :r.n_metrics], o1["metrics"][0, :r1.n_metrics],
                                      err_msg=f"patch {p} metric history")
        np.testing.assert_array_equal(out["alpha"][p][:I, :M], o1["alpha"][0], err_msg=f"patch {p} alpha")
        assert not out["alpha"][p][I:].any() and not out["alpha"][p][:, M:].any(), p
        np.testing.assert_array_equal(obj[p], obj1[0], err_msg=f"patch {p} restored objects")
    rs.close()


def test_ragged_rejections():
    c = CASES["fused88"]
    big, jobs, own, packed = _case(**c)
    s = S.Solver(big, max_patches=6)
    with pytest.raises(S.SolverError, match="patch shape 0"):
        s.set_patch_shapes([(9, 36, jobs[0].nullspace)], [0])            # more frames than the handle
    s.set_patch_shapes([(F, M, j.nullspace) for (F, M), j in zip(c["shapes"], jobs)], c["assign"])
    with pytest.raises(S.SolverError, match="given for 6 patches"):
        s.set_patches(packed[:3])
    with pytest.raises(S.SolverError, match="REG_ALPHA"):
        s.set_reg_alpha(np.ones((big.n_images, big.n_modes)))
    s.set_patch_shapes([], [])                                            # uniform again
    with pytest.raises(S.SolverError, match="non-finite regularisation"):
        s.set_patches(packed[:3])         # the unused slots are now images: blank ones
    s.set_patches(synth.make_patches(big, 3, 12.0, np.random.default_rng(3)).cutouts)
    s.close()
