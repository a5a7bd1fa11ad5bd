"""Python mirror of the library's once-per-job set-up (rdxg_setup.cpp through the C ABI):
pupil sampling, the anti-aliased pupil and its supports, Zernike and Karhunen-Loeve mode sets
and the apodisation windows, the static inputs redux computes once per job (GlobalData).
Host code only; no GPU is needed."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


def _check(r: int, what: str):
    if r != _lib.RDXG_OK:
        raise ValueError(f"{what}: status {r}")


def pupil_size(n_pixels: int, wavelength: float, telescope_d: float, arcsec_per_pixel: float):
    """(frequency_cutoff, radius_in_pixels, pupil_pixels): Pupil::calculatePupilSize."""
    L = _lib.load()
    fc, r, n = C.c_double(), C.c_double(), C.c_int32()
    _check(L.rdxg_pupil_size(n_pixels, wavelength, telescope_d, arcsec_per_pixel, C.byref(fc), C.byref(r),
                             C.byref(n)), "rdxg_pupil_size")
    return fc.value, r.value, n.value


def make_pupil(n: int, radius: float, inner_radius: float = 0.0):
    """(pupil [n, n], area): makePupil + Pupil::normalize."""
    L = _lib.load()
    out = np.zeros((n, n))
    area = C.c_double()
    _check(L.rdxg_make_pupil(n, radius, inner_radius, _lib.ptr(out), C.byref(area)), "rdxg_make_pupil")
    return out, area.value


def pupil_support(pupil: np.ndarray, threshold: float = 1e-9):
    """(pupil_support, pupil_in_otf, otf_support, area): Pupil::generateSupport."""
    L = _lib.load()
    p = np.ascontiguousarray(pupil, np.float64)
    n = p.shape[0]
    ps = np.zeros(n * n, np.int32)
    pin = np.zeros(n * n, np.int32)
    os_ = np.zeros(4 * n * n, np.int32)
    nps, nos, area = C.c_int32(), C.c_int32(), C.c_double()
    _check(L.rdxg_pupil_support(_lib.ptr(p), n, threshold, _lib.ptr(ps), C.byref(nps), _lib.ptr(pin), _lib.ptr(os_),
                                C.byref(nos), C.byref(area)), "rdxg_pupil_support")
    return ps[:nps.value].copy(), pin[:nps.value].copy(), os_[:nos.value].copy(), area.value


def make_modes(mode_list, n_pixels: int, radius: float, wavelength: float, jacobian_scale: float,
               kind: str = "zernike", angle: float = 0.0, kl_first: int = 2, kl_last: int = 2000,
               kl_cutoff: float = 1e-3):
    """(modes [M, n, n], atm_rms [M], J_T_xy [2, 2]): ModeSet::generate + normalize + measureJacobian."""
    L = _lib.load()
    ml = np.ascontiguousarray(mode_list, np.int32)
    M = ml.shape[0]
    prm = _lib.ModeParams(1 if kind == "kl" else 0, n_pixels, radius, wavelength, angle, jacobian_scale,
                          kl_first, kl_last, kl_cutoff)
    modes = np.zeros((M, n_pixels, n_pixels))
    atm = np.zeros(M)
    J = np.zeros((2, 2))
    _check(L.rdxg_make_modes(C.byref(prm), _lib.ptr(ml), M, _lib.ptr(modes), _lib.ptr(atm), _lib.ptr(J)),
           "rdxg_make_modes")
    return modes, atm, J


def apodization_windows(patch_size: int, apodization: int = -1):
    """(window, noise_window): Solver::init's apodised windows."""
    L = _lib.load()
    w = np.zeros((patch_size, patch_size))
    nw = np.zeros((patch_size, patch_size))
    _check(L.rdxg_apodization_windows(patch_size, apodization, _lib.ptr(w), _lib.ptr(nw)), "rdxg_apodization_windows")
    return w, nw
