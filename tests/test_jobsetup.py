"""Job set-up: pupil, supports, modes, constraints and the null-space map."""
import numpy as np
import pytest

from redux_gb300 import jobsetup as js
from redux_gb300 import synth


def test_pupil_size_critical_sampling():
    for N in (64, 88, 128):
        fc, r, n = js.calculate_pupil_size(N, synth.WAVELENGTH, synth.TELESCOPE_D, synth.ARCSEC_PER_PX)
        assert n == N // 2 and abs(r - N / 4) < 1e-9


def test_pupil_and_supports():
    p, area = js.make_pupil(32, 16.0)
    assert p.min() == 0.0 and p.max() == 1.0
    sup = js.pupil_support(p)
    assert abs(sup.area - p[p > 1e-9].sum()) < 1e-12
    N = 64
    # the OTF support is symmetric about the centre (lags u and -u)
    m = np.zeros(N * N, bool); m[sup.otf_support] = True; m = m.reshape(N, N)
    assert np.array_equal(m[1:, 1:], m[1:, 1:][::-1, ::-1])
    # pupilInOTF: the pupil embedded at offset n/2
    q = sup.pupil_support[0]
    assert sup.pupil_in_otf[0] == (q // 32) * N + q % 32 + 16 + 16 * N


def test_zernike_normalisation_and_tilt_jacobian():
    w = synth.make_job(64, 20, synth.LAYOUT_1OBJ(4))
    A = w.pupil
    for m in range(w.n_modes):
        z = w.modes[m] * w.wavelength
        np.testing.assert_allclose((z * z * A)[A > 0].sum() / w.support.area, 1.0, rtol=1e-10)
    assert w.tilt_x == 0 and w.tilt_y == 1
    J = w.J_T_xy
    assert abs(J[0, 0]) > 1e3 * abs(J[0, 1]) and abs(J[1, 1]) > 1e3 * abs(J[1, 0])


@pytest.mark.parametrize("frames,objects", [(4, [[0.0, 1.0]]), (12, [[0.0], [0.0, 1.0]]), (3, [[0.0, 1.0, 0.5]])])
def test_nullspace(frames, objects):
    wf, ref = [], []
    for o, chans in enumerate(objects):
        for c in range(len(chans)):
            for t in range(frames):
                if o == 0 and c == 0:
                    ref.append(len(wf))
                wf.append(t)
    M = 10
    ns = js.build_constraints(wf, M, ref)
    I = len(wf)
    C = len(wf) // frames
    # Constraints::init: (C - 1) equalities per wavefront and mode, plus one tilt sum per tilt mode
    n_con = M * frames * (C - 1) + 2
    assert ns.n_parameters == I * M
    assert ns.n_free == I * M - n_con
    Nm = ns.dense()
    np.testing.assert_allclose(Nm.T @ Nm, np.eye(ns.n_free), atol=1e-12)   # orthonormal
    # every column satisfies the constraints
    a = Nm @ np.random.default_rng(0).standard_normal(ns.n_free)
    a = a.reshape(I, M)
    for m in range(M):
        for t in range(frames):
            v = a[[j for j in range(I) if wf[j] == t], m]
            assert np.ptp(v) < 1e-12
    for m in (0, 1):
        assert abs(a[ref, m].sum()) < 1e-12


def test_kl_expansion_diagonalises_the_noll_covariance():
    from redux_gb300 import jobsetup as J
    first, last = 2, 73
    kle = J.kl_expansion(first, last)
    ids = list(range(first, last + 1))
    W = np.zeros((len(ids), len(ids)))
    for a, i in enumerate(ids):
        for j, c in kle[i].weights:
            W[a, j - first] = c
    C = np.array([[J.zernike_covariance(i, j) for j in ids] for i in ids])
    K = W @ C @ W.T
    assert np.abs(K - np.diag(np.diag(K))).max() <= 1e-12 * np.abs(np.diag(K)).max()
    np.testing.assert_allclose(np.diag(K), [kle[i].covariance for i in ids], rtol=1e-10)
    # each KL mode mixes only Zernikes of one azimuthal order and parity (one covariance block)
    for i in ids:
        ms = {abs(J.noll_to_nm(j)[1]) for j, c in kle[i].weights if abs(c) > 1e-12}
        assert len(ms) == 1
        # sign rule of the reference: the largest weight is positive
        cs = np.array([c for _, c in kle[i].weights])
        assert cs[np.argmax(np.abs(cs))] > 0


def test_kl_modeset_tilts_stay_zernike_and_modes_have_unit_rms():
    from redux_gb300 import jobsetup as J
    lam = 630.2e-9
    mode_list = list(range(2, 22))
    kl = J.kl_modeset(mode_list, 32, 16.0, lam, 1.0, 2, 41)
    zn = J.zernike_modeset(mode_list, 32, 16.0, lam, 1.0)
    np.testing.assert_allclose(kl.modes[0], zn.modes[0])   # Noll 2
    np.testing.assert_allclose(kl.modes[1], zn.modes[1])   # Noll 3
    pupil, _ = J.make_pupil(32, 16.0)
    area = J.pupil_support(pupil).area
    for m in kl.modes:
        rms = np.sqrt(((m * lam) ** 2 * pupil)[pupil > 0].sum() / area)
        assert abs(rms - 1.0) < 1e-12
    # KL mode 4 is dominated by defocus
    k = J.kl_expansion(2, 41)[4]
    assert max(k.weights, key=lambda t: abs(t[1]))[0] == 4
