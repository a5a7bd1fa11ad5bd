"""rdxg_metric_noalloc (the metric with its temporaries in the library's static device scratch)
against rdxg_metric, two calls in a row, and the size limit.  Named to be collected last, so
it also runs after every other test has used the library in the same process."""
import numpy as np
import pytest

from redux_gb300 import solver as S
from tests.conftest import workload

pytestmark = pytest.mark.gpu

# Same kernels and summation order as rdxg_metric, but both refresh the handle's reference
# object starting from its previous value, so two evaluations at one point (by either entry
# point) agree to the rounding of the FP32 accumulation (1e-10 ... 3e-8 measured), not bit for
# bit; the metric itself is within 1e-5 of FP64.
TOL = 1e-6


def _solver(w):
    P = w.patches.cutouts.shape[0]
    s = S.Solver(w.job, max_patches=P, precision="fp32")
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    return s


@pytest.mark.parametrize("cfg", ["plain64", "production88"])
def test_noalloc_matches_metric_two_calls(cfg):
    w = workload("plain64") if cfg == "plain64" else workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    for scale in (0.5, 1.0):
        a = w.patches.alpha_true * scale
        ref = s.metric(a)
        first = s.metric_noalloc(a)
        second = s.metric_noalloc(a)
        np.testing.assert_allclose(first, ref, rtol=TOL, atol=0)
        np.testing.assert_allclose(second, ref, rtol=TOL, atol=0)
        np.testing.assert_allclose(second, first, rtol=TOL, atol=0)


def _free_device_bytes():
    # cudaMemGetInfo of the current device (torch.cuda.mem_get_info); the test makes no torch
    # allocation in between
    import torch
    free, _ = torch.cuda.mem_get_info()
    return free


def test_noalloc_allocates_nothing():
    """The entry point's defining property: neither the handle nor the device gains memory over
    its first and second call (the static scratch is reserved when the handle is created)."""
    w = workload("production88", n_patches=2, frames=4)
    s = _solver(w)
    a = w.patches.alpha_true * 0.5
    n0 = int(s.debug("allocations")[0])
    free0 = _free_device_bytes()
    first = s.metric_noalloc(a)
    second = s.metric_noalloc(a)
    free1 = _free_device_bytes()
    assert int(s.debug("allocations")[0]) == n0
    assert free1 == free0, (free0, free1)
    np.testing.assert_allclose(second, first, rtol=TOL, atol=0)


def test_noalloc_rejects_batches_beyond_the_scratch():
    # 88 x 88, 12 images per patch: about 255 KB of temporaries per patch, 70 patches > 16 MiB
    w = workload("production88", n_patches=70, frames=4)
    s = _solver(w)
    with pytest.raises(S.SolverError, match="static scratch holds"):
        s.metric_noalloc(w.patches.alpha_true)
    # the handle stays usable
    assert np.all(np.isfinite(s.metric(w.patches.alpha_true)))
    # and a batch that fits still agrees with rdxg_metric
    small = workload("production88", n_patches=2, frames=4)
    s2 = _solver(small)
    np.testing.assert_allclose(s2.metric_noalloc(small.patches.alpha_true), s2.metric(small.patches.alpha_true),
                               rtol=TOL, atol=0)
