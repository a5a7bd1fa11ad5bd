"""Known-answer tests of the oracle's FFT conventions, restated from the reference's
testsuite/image/fourier.cpp (forward transforms 226-320, reorder 396-460, autocorrelation
845-911).  They pin the DFT sign, normalisation and centring the whole solver relies on."""
import numpy as np
import pytest

import oracle

TOL = 1e-9


@pytest.mark.parametrize("ny,nx", [(64, 64), (64, 63), (64, 53), (53, 71), (88, 88), (88, 53)])
def test_forward_constant_and_delta(ny, nx):
    ones = np.ones((ny, nx))
    ft = oracle.fft2(ones)
    exp = np.zeros((ny, nx), complex)
    exp[0, 0] = nx * ny                          # DC not normalised by default
    assert np.abs(ft - exp).max() < TOL * nx * ny
    # REORDER_FT puts DC at (ny/2, nx/2)
    c = oracle.reorder(ft)
    exp = np.zeros((ny, nx), complex)
    exp[ny // 2, nx // 2] = nx * ny
    assert np.abs(c - exp).max() < TOL * nx * ny
    # NORMALIZE_FT divides by the number of pixels
    assert abs(ft[0, 0] / (nx * ny) - 1.0) < TOL
    # a delta at (0, 0) transforms to a constant 1
    d = np.zeros((ny, nx)); d[0, 0] = 1
    assert np.abs(oracle.fft2(d) - 1.0).max() < TOL


@pytest.mark.parametrize("n", [64, 88])
def test_forward_cosines(n):
    y, x = np.mgrid[0:n, 0:n]
    f = np.cos(y * 2.0 * np.pi / n) + np.cos(x * 4.0 * np.pi / n)
    ft = oracle.reorder(oracle.fft2(f)) / (n * n)
    exp = np.zeros((n, n))
    exp[n // 2 + 1, n // 2] = exp[n // 2 - 1, n // 2] = 0.5
    exp[n // 2, n // 2 + 2] = exp[n // 2, n // 2 - 2] = 0.5
    assert np.abs(ft - exp).max() < 1e-12


def test_inverse_round_trip():
    rng = np.random.default_rng(1)
    a = rng.standard_normal((88, 88)) + 1j * rng.standard_normal((88, 88))
    b = oracle.fft2(oracle.fft2(a, -1), +1) / (88 * 88)
    assert np.abs(a - b).max() < 1e-12
    np.testing.assert_allclose(oracle.fft2(a), np.fft.fft2(a), atol=1e-10)


def test_reorder_layouts():
    inp = np.arange(1, 101, dtype=float)
    out = oracle.reorder_into(inp[:16].reshape(4, 4))
    np.testing.assert_array_equal(out.ravel(), [11, 12, 9, 10, 15, 16, 13, 14, 3, 4, 1, 2, 7, 8, 5, 6])
    np.testing.assert_array_equal(oracle.reorder_into(out).ravel(), inp[:16])     # even: own inverse
    out = oracle.reorder_into(inp[:25].reshape(5, 5))
    np.testing.assert_array_equal(out.ravel(), [19, 20, 16, 17, 18, 24, 25, 21, 22, 23, 4, 5, 1, 2, 3,
                                                9, 10, 6, 7, 8, 14, 15, 11, 12, 13])
    out = oracle.reorder_into(inp[:16].reshape(4, 4), (5, 6))
    np.testing.assert_array_equal(out.ravel(), [11, 12, 0, 0, 9, 10, 15, 16, 0, 0, 13, 14, 0, 0, 0, 0, 0, 0,
                                                3, 4, 0, 0, 1, 2, 7, 8, 0, 0, 5, 6])
    out = oracle.reorder_into(inp[:16].reshape(4, 4), (5, 6), center=True)
    np.testing.assert_array_equal(out.ravel(), [0, 11, 12, 9, 10, 0, 0, 15, 16, 13, 14, 0, 0, 3, 4, 1, 2, 0,
                                                0, 7, 8, 5, 6, 0, 0, 0, 0, 0, 0, 0])
    with pytest.raises(ValueError):
        oracle.reorder_into(inp[:16].reshape(4, 4), (3, 4))
    # the in-place reorder used by the solver equals reorderInto
    a = np.arange(88 * 88, dtype=float).reshape(88, 88)
    np.testing.assert_array_equal(oracle.reorder(a), oracle.reorder_into(a))


def test_autocorrelation_kat():
    n = 64
    a = np.zeros((n, n))
    a[5, 5] = a[6, 6] = a[6, 5] = a[5, 6] = 3
    exp = np.zeros((n, n))
    exp[0, 0] = 36
    exp[0, 1] = exp[1, 0] = exp[n - 1, 0] = exp[0, n - 1] = 18
    exp[1, 1] = exp[n - 1, n - 1] = exp[n - 1, 1] = exp[1, n - 1] = 9
    assert np.abs(oracle.autocorrelate(a, center=False) - exp).max() < 1e-10
    assert np.abs(oracle.autocorrelate(a, center=True) - oracle.reorder(exp)).max() < 1e-10
