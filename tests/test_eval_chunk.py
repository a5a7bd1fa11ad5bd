"""Images per work item of the fused evaluation (rdxg_geometry.eval_chunk): the value changes the
grouping of the chunk sums (FP32 rounding) and nothing else, and a patch's results depend on it
and on nothing else of the batch, so the split used by the benchmark (several handles, one work
item per object) solves every patch as one handle of the whole batch does (marked gpu)."""
import numpy as np
import pytest

from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def w12():
    # the production geometry: 88 x 88, 36 modes, 3 channels x 12 frames, objects of 12 and 24
    # images (the wide-band channel; the two narrow-band channels)
    return workload("production88", n_patches=6, frames=12)


def _solver(w, chunk, sl=slice(None)):
    cut = w.patches.cutouts[sl]
    s = S.Solver(w.job, max_patches=cut.shape[0], eval_chunk=chunk)
    s.set_patches(cut)
    return s


def test_chunk_sizes_agree_to_fp32_rounding(w12):
    a = w12.patches.alpha_true
    ref = _solver(w12, 0)
    L0, (g0, _) = ref.metric(a), ref.gradient(a)
    for chunk in (1, 9, 18, 32):
        s = _solver(w12, chunk)
        L, (g, _) = s.metric(a), s.gradient(a)
        # metric: relative 1e-6 (FP32 sums of up to 24 images per point, added in another grouping)
        np.testing.assert_allclose(L, L0, rtol=1e-6, atol=0)
        for p in range(a.shape[0]):
            assert np.linalg.norm(g[p] - g0[p]) <= 1e-5 * np.linalg.norm(g0[p]), (chunk, p)
        s.close()
    ref.close()


def test_one_item_per_object_split_over_handles_equals_one_handle(w12):
    st = S.fixed_iterations(w12.job.n_modes, 6, max_metrics=96)
    whole = _solver(w12, 18)
    alone = whole.run(st)
    parts = [_solver(w12, 18, slice(k, k + 2)) for k in (0, 2, 4)]
    together = S.solve_many(parts, st)
    alpha = np.concatenate([t["alpha"] for t in together])
    np.testing.assert_array_equal(alpha, alone["alpha"])
    reps = [r for t in together for r in t["reports"]]
    for p, r in enumerate(reps):
        b = alone["reports"][p]
        assert (r.n_metrics, r.iterations, r.final_metric) == (b.n_metrics, b.iterations, b.final_metric)
    for s in parts + [whole]:
        s.close()
