"""The launch-shape planner (rdxg_autotune): every compiled block size of k_eval, k_forward
and k_adjoint gives bit-identical metrics, gradients and solves, so the planner may pick any
of them by speed alone (marked gpu)."""
import numpy as np
import pytest

from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu

# k_eval: 512 or 384 threads
EVAL_ALT = 384

# (workload, shapes to compare): the fused path (64, 88) tunes k_eval and k_adjoint, the
# general path (128) k_forward and k_adjoint.  fused88batch gives every block of the
# evaluation several work items (chunks of several objects and patches), with gradient
# evaluations among them.
CASES = {
    "fused64": (lambda: workload("plain64"), [dict(eval_threads=512, adjoint_threads=256),
                                      dict(eval_threads=EVAL_ALT, adjoint_threads=512)]),
    "fused88": (lambda: workload("production88", n_patches=2, frames=4), [dict(eval_threads=512, adjoint_threads=256),
                                                             dict(eval_threads=EVAL_ALT, adjoint_threads=512)]),
    "fused88batch": (lambda: workload("production88", n_patches=64, frames=12),
                     [dict(eval_threads=512, adjoint_threads=256), dict(eval_threads=EVAL_ALT, adjoint_threads=512)]),
    "general128": (lambda: workload("large128", n_patches=1, frames=2), [dict(forward_threads=512, adjoint_threads=512),
                                                                dict(forward_threads=1024, adjoint_threads=1024)]),
}


def _run(w, shape):
    P = w.patches.cutouts.shape[0]
    s = S.Solver(w.job, max_patches=P)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    if shape is not None:
        s.set_launch_shape(**shape)
    a = w.patches.alpha_true * 0.5
    L = s.metric(a)
    g, _ = s.gradient(a, "vogel")
    out = s.run(S.fixed_iterations(w.job.n_modes, 3, max_metrics=16))
    got = s.launch_shape()
    s.close()
    return L, g, out, got


@pytest.mark.parametrize("case", sorted(CASES))
def test_every_shape_gives_identical_results(case):
    make, shapes = CASES[case]
    w = make()
    ref = None
    for sh in shapes:
        L, g, out, got = _run(w, sh)
        for k, v in sh.items():
            assert got[k.replace("_threads", "")] == v, (got, sh)
        if ref is None:
            ref = (L, g, out)
            ref_radix = {k: got[k + "_radix"] for k in ("eval", "forward", "adjoint")}
            continue
        np.testing.assert_array_equal(L, ref[0])
        np.testing.assert_array_equal(g, ref[1])
        np.testing.assert_array_equal(out["alpha"], ref[2]["alpha"])
        np.testing.assert_array_equal(out["metrics"], ref[2]["metrics"])
    # the planner on the first solve picks one of them: the results stay the same (unless it
    # also picked the other radix plan, whose rounding differs; see test_radix_plans)
    L, g, out, got = _run(w, None)
    if all(got[k + "_radix"] == ref_radix[k] for k in ("eval", "forward", "adjoint")):
        np.testing.assert_array_equal(out["alpha"], ref[2]["alpha"])


@pytest.mark.parametrize("case", sorted(CASES))
def test_autotune_reports_the_candidates(case):
    make, shapes = CASES[case]
    w = make()
    s = S.Solver(w.job, max_patches=w.patches.cutouts.shape[0])
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    r = s.autotune(reps=2)
    fused = case.startswith("fused")
    tuned = ("eval", "adjoint") if fused else ("forward", "adjoint")
    for k in tuned:
        assert all(t > 0 for t in r["ms"][k]), r
        allowed = {sh[k + "_threads"] for sh in shapes}
        assert r["shape"][k] in allowed, r
        # the faster candidate is kept (shapes[0]: the defaults, shapes[1]: the alternatives)
        faster = shapes[0] if r["ms"][k][0] <= r["ms"][k][1] else shapes[1]
        assert r["shape"][k] == faster[k + "_threads"], r
    untuned = "forward" if fused else "eval"
    assert r["shape"][untuned] == 0 and r["ms"][untuned] == [0.0, 0.0], r
    with pytest.raises(S.SolverError, match="not compiled"):
        s.set_launch_shape(adjoint_threads=300)
    with pytest.raises(S.SolverError, match="not used on this handle's path"):
        s.set_launch_shape(**{untuned + "_threads": 512})
    s.close()


def test_fp64_has_one_shape():
    w = workload("plain64")
    s = S.Solver(w.job, max_patches=1, precision="fp64")
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    r = s.autotune(reps=1)
    assert {k: r["shape"][k] for k in ("eval", "forward", "adjoint")} == dict(eval=0, forward=256, adjoint=256), r
    with pytest.raises(S.SolverError, match="not compiled"):
        s.set_launch_shape(adjoint_threads=512)
    s.close()


# the radix plans of the sizes that have two (32, 64: k_eval and k_adjoint; 128: k_forward and
# k_adjoint): the same transforms rounded differently
RADIX = {
    "fused64": (lambda: workload("plain64"), dict(eval_radix=8, adjoint_radix=8), dict(eval_radix=16, adjoint_radix=16)),
    "general128": (lambda: workload("large128", n_patches=1, frames=2), dict(forward_radix=16, adjoint_radix=16),
                   dict(forward_radix=8, adjoint_radix=8)),
}


@pytest.mark.parametrize("case", sorted(RADIX))
def test_radix_plans(case):
    make, p0, p1 = RADIX[case]
    w = make()
    out = []
    for plan in (p0, p1):
        s = S.Solver(w.job, max_patches=w.patches.cutouts.shape[0])
        s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
        s.set_launch_shape(**plan)
        got = s.launch_shape()
        for k, v in plan.items():
            assert got[k] == v, (got, plan)
        a = w.patches.alpha_true * 0.5
        out.append((s.metric(a), s.gradient(a, "vogel")[0]))
        s.close()
    (L0, g0), (L1, g1) = out
    np.testing.assert_allclose(L1, L0, rtol=1e-6)
    assert np.linalg.norm(g1 - g0) / np.linalg.norm(g0) < 1e-5
    s = S.Solver(w.job, max_patches=1)
    with pytest.raises(S.SolverError, match="not a plan"):
        s.set_launch_shape(adjoint_radix=5)
    s.close()
