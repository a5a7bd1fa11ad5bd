"""The CPU baseline's transform (oracle.set_fast_fft(True): iterative Stockham stages with
precomputed tables) against the oracle's own recursive FFT and numpy, and a patch's metric and
gradient with each (CPU only).  The fast form is only timed, never used as the checker; this
keeps what is timed the same computation."""
import numpy as np
import pytest

import oracle


@pytest.fixture
def fast():
    oracle.set_fast_fft(True)
    yield
    oracle.set_fast_fft(False)


@pytest.mark.parametrize("n", [32, 64, 88, 128, 44, 96])
@pytest.mark.parametrize("sign", [-1, +1])
def test_fast_transform_equals_the_recursive_one(n, sign):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    slow = oracle.fft2(a, sign)
    oracle.set_fast_fft(True)
    try:
        quick = oracle.fft2(a, sign)
    finally:
        oracle.set_fast_fft(False)
    want = np.fft.fft2(a) if sign < 0 else np.fft.ifft2(a) * n * n
    scale = np.abs(want).max()
    assert np.abs(quick - want).max() <= 1e-13 * scale
    assert np.abs(quick - slow).max() <= 1e-13 * scale


def test_fast_transform_metric_and_gradient_match(fast):
    # the metric and the Vogel gradient of a patch at the true coefficients with each transform
    # (a solve's trajectory amplifies the transforms' different rounding, as any change of
    # rounding does, so the comparison is at fixed points)
    from tests.conftest import workload
    w = workload("production88", n_patches=1, frames=4)
    a = w.patches.alpha_true[0]
    op = oracle.OraclePatch(w.job, threads=1)
    op.set_images(w.patches.cutouts[0], None, None)
    lq, gq = op.metric(a), op.gradient(a)[1]
    oracle.set_fast_fft(False)
    op2 = oracle.OraclePatch(w.job, threads=1)
    op2.set_images(w.patches.cutouts[0], None, None)
    ls, gs = op2.metric(a), op2.gradient(a)[1]
    np.testing.assert_allclose(lq, ls, rtol=1e-10)
    assert np.linalg.norm(gq - gs) <= 1e-8 * np.linalg.norm(gs)
