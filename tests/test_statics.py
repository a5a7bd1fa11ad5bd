"""The library's once-per-job set-up (rdxg_setup.cpp: rdxg_pupil_size, rdxg_make_pupil,
rdxg_pupil_support, rdxg_make_modes, rdxg_apodization_windows) against the numpy restatement
that builds the test and benchmark jobs (redux_gb300/jobsetup.py): pupil sampling
(pupil.cpp:78-100), makePupil (image/utils.cpp:68-124), Pupil::generateSupport
(pupil.cpp:245-277), Zernike and Karhunen-Loeve ModeSets with their normalisation and tilt
Jacobian (modes.cpp:158-197, 348-535; zernike.cpp:69-479), Solver::init's windows
(solver.cpp:113-126).  Host code, run on the CPU."""
import math

import numpy as np
import pytest

from redux_gb300 import jobsetup as J
from redux_gb300 import statics, synth


@pytest.mark.parametrize("N", [64, 88, 128])
def test_pupil_size(N):
    got = statics.pupil_size(N, synth.WAVELENGTH, synth.TELESCOPE_D, synth.ARCSEC_PER_PX)
    want = J.calculate_pupil_size(N, synth.WAVELENGTH, synth.TELESCOPE_D, synth.ARCSEC_PER_PX)
    assert got[2] == want[2]
    np.testing.assert_allclose(got[:2], want[:2], rtol=1e-15)


@pytest.mark.parametrize("n,radius,inner", [(32, 16.0, 0.0), (44, 22.0, 0.0), (64, 32.0, 0.0), (44, 21.3, 5.2)])
def test_pupil_and_supports(n, radius, inner):
    p, area = statics.make_pupil(n, radius, inner)
    pp, aa = J.make_pupil(n, radius, inner)
    np.testing.assert_allclose(p, pp, rtol=0, atol=1e-15)
    assert abs(area - aa) <= 1e-12 * aa
    ps, pin, osup, sarea = statics.pupil_support(p)
    want = J.pupil_support(pp)
    np.testing.assert_array_equal(ps, want.pupil_support)
    np.testing.assert_array_equal(pin, want.pupil_in_otf)
    np.testing.assert_array_equal(osup, want.otf_support)
    assert abs(sarea - want.area) <= 1e-12 * want.area


def _jscale(N):
    fc, _, _ = J.calculate_pupil_size(N, synth.WAVELENGTH, synth.TELESCOPE_D, synth.ARCSEC_PER_PX)
    return synth.WAVELENGTH * (0.5 * fc) / ((math.pi * math.pi / 648000.0) * synth.ARCSEC_PER_PX * synth.TELESCOPE_D)


def _check_modes(got, want, rtol=1e-12):
    modes, atm, Jt = got
    scale = np.abs(want.modes).max()
    assert np.abs(modes - want.modes).max() <= rtol * scale
    np.testing.assert_allclose(atm, want.atm_rms, rtol=1e-12)
    # the tilt Jacobian: the off-diagonal entries are rounding residue of the plane fits
    jm = np.abs(want.J_T_xy).max()
    assert np.abs(Jt - want.J_T_xy).max() <= 1e-12 * jm


def test_zernike_modeset_64():
    ml = list(range(2, 22))    # the plain 64 x 64 job: Zernike 2-21
    _check_modes(statics.make_modes(ml, 32, 16.0, synth.WAVELENGTH, _jscale(64)),
                 J.zernike_modeset(ml, 32, 16.0, synth.WAVELENGTH, _jscale(64)))


@pytest.mark.parametrize("N,M", [(88, 36), (128, 100)])
def test_kl_modeset(N, M):
    # the production and large jobs: KL 2..M+1 (tilts Zernike) over Noll 2..2M+1
    _, radius, npup = J.calculate_pupil_size(N, synth.WAVELENGTH, synth.TELESCOPE_D, synth.ARCSEC_PER_PX)
    ml = list(range(2, 2 + M))
    got = statics.make_modes(ml, npup, radius, synth.WAVELENGTH, _jscale(N), kind="kl", kl_first=2, kl_last=2 * M + 1)
    want = J.kl_modeset(ml, npup, radius, synth.WAVELENGTH, _jscale(N), 2, 2 * M + 1)
    # the high KL modes of the 100-mode set mix Zernikes up to radial order ~18, whose
    # polynomial sums cancel (coefficients up to ~1e8): the two restatements' roundings
    # (repeated products against pow, Jacobi rotations against LAPACK's SVD) part at ~3e-12
    _check_modes(got, want, rtol=1e-12 if M <= 36 else 1e-10)


def test_modes_match_the_synthetic_job():
    # the static inputs of a benchmark job, as the library would produce them for rdxg_create
    w = synth.workload("production88", n_patches=1, frames=2)
    job = w.job
    _, radius, _ = J.calculate_pupil_size(88, synth.WAVELENGTH, synth.TELESCOPE_D, synth.ARCSEC_PER_PX)
    modes, _, Jt = statics.make_modes(job.mode_list, job.pupil_pixels, radius, synth.WAVELENGTH, _jscale(88),
                                      kind="kl", kl_last=2 * job.n_modes + 1)
    assert np.abs(modes - job.modes).max() <= 1e-12 * np.abs(job.modes).max()
    p, _ = statics.make_pupil(job.pupil_pixels, radius)
    np.testing.assert_allclose(p, job.pupil, atol=1e-15)
    win, nwin = statics.apodization_windows(88)
    np.testing.assert_array_equal(win, job.window)
    np.testing.assert_array_equal(nwin, job.noise_window)


@pytest.mark.parametrize("size,apod", [(64, -1), (88, -1), (88, 0), (128, 20)])
def test_windows(size, apod):
    w, nw = statics.apodization_windows(size, apod)
    ww, nww = J.solver_windows(size, apod)
    np.testing.assert_array_equal(w, ww)
    np.testing.assert_array_equal(nw, nww)


def test_rejects_bad_arguments():
    with pytest.raises(ValueError):
        statics.make_modes([1, 2], 32, 16.0, synth.WAVELENGTH, 1.0)        # piston is not a mode here
    with pytest.raises(ValueError):
        statics.make_modes([2, 3, 80], 32, 16.0, synth.WAVELENGTH, 1.0, kind="kl", kl_last=40)
    with pytest.raises(ValueError):
        statics.pupil_size(2, synth.WAVELENGTH, synth.TELESCOPE_D, synth.ARCSEC_PER_PX)
