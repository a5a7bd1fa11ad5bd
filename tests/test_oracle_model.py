"""The C oracle against an independent numpy restatement, and the gradient relations."""
import numpy as np
import pytest

import oracle
from oracle.np_oracle import NumpyModel
from tests.conftest import workload


def _pair(w, p=0):
    op = oracle.OraclePatch(w.job)
    fg = None if w.patches.fixed_gamma is None else w.patches.fixed_gamma[p]
    op.set_images(w.patches.cutouts[p], None, fg)
    nm = NumpyModel(w.job, op.D(), op.gamma(), op.otfnorm())
    return op, nm


@pytest.mark.parametrize("scale", [0.0, 0.5, 1.0])
def test_metric_matches_numpy(w0, scale):
    op, nm = _pair(w0)
    a = w0.patches.alpha_true[0] * scale
    L = op.metric(a)
    assert abs(L - nm.metric(a)) <= 1e-11 * abs(L)


def test_otf_normalisation(w0):
    op, _ = _pair(w0)
    op.metric(np.zeros((w0.job.n_images, w0.job.n_modes)))
    S = op.otf()
    N = w0.job.otf_size
    # S(0) = 1 for every image (Channel::initPatch normalisation, channel.cpp:941-952)
    np.testing.assert_allclose(S[:, N // 2, N // 2].real, 1.0, atol=1e-12)


@pytest.mark.parametrize("kind", ["vogel", "exact"])
def test_gradient_matches_numpy(w0, kind):
    op, nm = _pair(w0)
    a = w0.patches.alpha_true[0] * 0.5
    gn = nm.gradient(a, kind)
    if kind == "vogel":
        _, go = op.gradient(a, "vogel")
        assert np.linalg.norm(go - gn) / np.linalg.norm(go) < 1e-10


def test_exact_gradient_is_the_derivative(w0):
    """Central differences of the oracle metric agree with the exact adjoint."""
    op, nm = _pair(w0)
    a = w0.patches.alpha_true[0] * 0.5
    ge = nm.gradient(a, "exact")
    h = 1e-4 * w0.job.wavelength
    gc = np.zeros((2, w0.job.n_modes))
    for j in range(2):
        for m in range(w0.job.n_modes):
            ap = a.copy(); ap[j, m] += h
            am = a.copy(); am[j, m] -= h
            gc[j, m] = (op.metric(ap) - op.metric(am)) / (2 * h)
    assert np.linalg.norm(ge[:2] - gc) / np.linalg.norm(gc) < 1e-6


def test_vogel_is_weighted_exact(w0):
    """The reference's gradient is the exact adjoint with the pupil amplitude as an extra
    per-pixel weight and the constant -2 area / N^2 (object weight applied twice)."""
    job = w0.job
    op, nm = _pair(w0)
    a = w0.patches.alpha_true[0] * 0.5
    _, gv = op.gradient(a, "vogel")
    ge = nm.gradient(a, "exact")
    ratio = (gv / ge).ravel()
    N, A = job.otf_size, job.pupil
    area = float(A.sum())
    c2 = 1.0 / float((A * A).sum())
    const = (2 * area / N ** 2) / (4 * c2 * N ** 2 / job.patch_size ** 2)
    # binary pupils would give exactly `const`; the anti-aliased rim spreads the ratio
    assert 0.2 * const < np.median(ratio) < 2.0 * const


def test_fd_gradient_close_to_central(w0):
    op, _ = _pair(w0)
    a = w0.patches.alpha_true[0] * 0.5
    _, gf = op.gradient(a, "fd")
    _, ge = None, NumpyModel(w0.job, op.D(), op.gamma(), op.otfnorm()).gradient(a, "exact")
    # one-sided differences with a 0.01 rad step: first-order accurate
    assert np.linalg.norm(gf - ge) / np.linalg.norm(ge) < 0.05


def test_noise_derived_gamma_positive(w2small):
    op, _ = _pair(w2small)
    g = op.gamma()
    assert np.all(g > 0) and np.all(np.isfinite(g))
