"""Host-side, once-per-job set-up of the static inputs of the per-patch solver.

These are the pieces that redux computes once per job on the master (and ships to
every worker in ``GlobalData``) before any patch is solved.  The per-patch solver
core in this package consumes them; it never recomputes them.

* pupil sampling and geometry  -- ``Pupil::calculatePupilSize`` (src/lib/image/pupil.cpp:78-100),
  ``makePupil`` (src/lib/image/utils.cpp:68-124), ``Pupil::normalize`` (pupil.cpp:280-300),
  ``Pupil::generateSupport`` (pupil.cpp:245-277)
* Zernike modes                -- ``Zernike::NollToNM`` (src/lib/image/zernike.cpp:69-80),
  ``Zernike::getZernike`` (zernike.cpp:234-274), ``ModeSet::getNorms``/``normalize``
  (src/lib/momfbd/modes.cpp:443-462, 524-535), ``GlobalData::get`` (src/lib/momfbd/data.cpp:658-686)
* tilt Jacobian                -- ``ModeSet::measureJacobian`` (modes.cpp:464-512),
  ``fitPlane`` (src/lib/image/utils.cpp:169-233)
* apodisation window           -- ``apodizeInPlace`` (utils.cpp:584-614), ``math::apodize``
  (src/lib/math/functions.cpp:39-50), ``Solver::init`` (src/lib/momfbd/solver.cpp:113-126)
* linear constraints           -- ``Constraints::init`` (src/lib/momfbd/constraints.cpp:536-622)

All arithmetic is float64 numpy.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

RADIANS_PER_ARCSEC = math.pi / (180.0 * 3600.0)
GOOD_SIZES = (16, 18, 20, 24, 25, 27, 30, 32, 36, 40, 45, 48, 50, 54, 60, 64, 72, 75, 80, 81,
              90, 96, 100, 108, 120, 125, 128, 135, 144)


def calculate_pupil_size(n_pixels: int, wavelength: float, telescope_d: float,
                         arcsec_per_pixel: float):
    """Returns (frequency_cutoff, pupil_radius_in_pixels, pupil_pixels).

    Restates Pupil::calculatePupilSize (src/lib/image/pupil.cpp:78-100)."""
    if n_pixels < 4:
        raise ValueError("n_pixels < 4")
    rad_per_px = arcsec_per_pixel * RADIANS_PER_ARCSEC
    q_number = wavelength / (rad_per_px * telescope_d)
    freq_cutoff = float(n_pixels) / q_number
    n_pup = n_pixels >> 2
    radius = freq_cutoff / 2.0
    if n_pup < radius:
        for gs in GOOD_SIZES:
            n_pup = max(gs, n_pup)
            if n_pup >= radius:
                break
    return freq_cutoff, radius, n_pup << 1


def _grid(n: int, origin_y: float, origin_x: float):
    """Grid::init (src/lib/image/grid.cpp:45-67): distance and angle of each pixel centre."""
    oy, ox = origin_y - 0.5, origin_x - 0.5
    y = np.arange(n, dtype=np.float64)[:, None] - oy
    x = np.arange(n, dtype=np.float64)[None, :] - ox
    dist = np.sqrt(y * y + x * x)
    ang = np.arctan2(y, x)
    at_origin = (y == 0) & (x == 0)
    dist = np.where(at_origin, 0.0, dist)
    ang = np.where(at_origin, 0.0, ang)
    return dist, ang


def make_pupil(n: int, radius: float, inner_radius: float = 0.0):
    """Anti-aliased annular aperture on an n x n grid centred on pixel (n/2, n/2).

    Restates makePupil (src/lib/image/utils.cpp:68-124) with the default centre of
    include/redux/image/utils.hpp:28-31, followed by Pupil::normalize (rescale to [0, 1]).
    Returns (pupil, area) where area is the makePupil sum."""
    mid = n / 2.0 + 0.5
    dist, ang = _grid(n, mid, mid)
    absang = np.abs(ang)
    with np.errstate(divide="ignore"):
        d = np.where((absang > math.pi / 4) & (absang < 3 * math.pi / 4),
                     np.abs(1.0 / np.sin(absang)), np.abs(1.0 / np.cos(absang)))
    has_inner = inner_radius > 0
    out = np.zeros((n, n))
    dir_ = dist - inner_radius
    dor = dist - radius
    for y in range(n):
        for x in range(n):
            dd = d[y, x]
            if has_inner and dir_[y, x] < -dd:
                continue
            if dor[y, x] > dd:
                continue
            if dor[y, x] < -dd and (not has_inner or dir_[y, x] > dd):
                out[y, x] = 1.0
                continue
            R = dor[y, x]
            dd2 = 2 * dd
            if has_inner and dor[y, x] < -dd2:
                R = dir_[y, x]
                dd2 = -dd2
            out[y, x] = 0.5 - R / dd2
    area = float(out.sum())
    mn, mx = out.min(), out.max()
    if mn != mx:
        out = (out - mn) / (mx - mn)
    return out, area


@dataclass
class PupilSupport:
    pupil_support: np.ndarray   # int32 flat indices into n*n where pupil > threshold
    pupil_in_otf: np.ndarray    # int32 flat indices into N*N (N = 2n)
    otf_support: np.ndarray     # int32 flat indices into the centred N*N OTF
    area: float                 # sum of the pupil over pupil_support


def pupil_support(pupil: np.ndarray, threshold: float = 1e-9) -> PupilSupport:
    """Pupil::generateSupport (src/lib/image/pupil.cpp:245-277)."""
    n = pupil.shape[0]
    N = 2 * n
    flat = pupil.ravel()
    sup = np.nonzero(flat > threshold)[0].astype(np.int32)
    area = float(flat[sup].sum())
    pin = ((sup // n) * N + (sup % n) + (n // 2) + (n // 2) * N).astype(np.int32)
    big = np.zeros((N, N))
    big[:n, :n] = pupil
    f = np.fft.fft2(big)
    ac = np.real(np.fft.ifft2(np.abs(f) ** 2))
    ac = np.fft.fftshift(ac)
    otf_sup = np.nonzero(np.abs(ac.ravel()) > threshold)[0].astype(np.int32)
    return PupilSupport(sup, pin, otf_sup, area)


def noll_to_nm(j: int):
    """Zernike::NollToNM (src/lib/image/zernike.cpp:69-80)."""
    n = 0
    length = 1
    i = 1
    while length < j:
        n = i
        length += n + 1
        i += 1
    dl = n + 1 - length + j
    m = 2 * ((dl + (n % 2)) // 2) + (0 if (n % 2) else 1) - 1
    if j % 2:
        m = -m
    return n, m


def zernike(j: int, n_pixels: int, radius: float, angle: float = 0.0) -> np.ndarray:
    """Zernike mode j (Noll) on the pupil grid, before the ModeSet normalisation.

    Follows Zernike::getZernike with the NORMALIZE flag (zernike.cpp:234-274): radial
    polynomial times cos/sin(m (theta - angle)), then scaled so that
    sum(Z^2 * pupil) == pupil area."""
    if j < 2:
        return np.full((n_pixels, n_pixels), float(j))
    nn, m = noll_to_nm(j)
    am = abs(m)
    mid = n_pixels / 2.0 + 0.5
    dist, ang = _grid(n_pixels, mid, mid)
    r = dist / radius
    R = np.zeros_like(r)
    for s in range((nn - am) // 2 + 1):
        c = ((-1) ** s * math.factorial(nn - s) /
             (math.factorial(s) * math.factorial((nn + am) // 2 - s) * math.factorial((nn - am) // 2 - s)))
        R += c * r ** (nn - 2 * s)
    if m > 0:
        Z = R * np.cos(am * (ang - angle))
    elif m < 0:
        Z = R * np.sin(am * (ang - angle))
    else:
        Z = R
    pupil, _ = make_pupil(n_pixels, radius)
    nrm = math.sqrt(pupil.sum() / float((Z * Z * pupil).sum()))
    return Z * nrm


def zernike_covariance(i: int, j: int) -> float:
    """Noll covariance of Zernike coefficients for Kolmogorov turbulence at D/r0 = 1.

    Restates Zernike::calcCovariance (src/lib/image/zernike.cpp:82-125)."""
    if i < 2 or j < 2:
        return 0.0
    n1, m1 = noll_to_nm(i)
    n2, m2 = noll_to_nm(j)
    if m1 != 0 and (i + j) % 2:
        return 0.0
    m1a, m2a = abs(m1), abs(m2)
    if m1a != m2a:
        return 0.0
    lg = math.lgamma
    k = ((4.8 * math.exp(lg(6.0 / 5.0))) ** (5.0 / 6.0) *
         math.exp(lg(14.0 / 3.0) + 2.0 * lg(11.0 / 6.0)) / (2.0 ** (8.0 / 3.0) * math.pi))
    k *= (-1.0) ** ((n1 + n2 - 2 * m1a) / 2.0) * math.sqrt((n1 + 1) * (n2 + 1))

    def sg(x):
        return math.copysign(1.0, math.gamma(x)) if x <= 0 and x != int(x) else 1.0

    a1 = ((n1 + n2) - 5.0 / 3.0) / 2.0
    a2 = ((n1 - n2) + 17.0 / 3.0) / 2.0
    a3 = ((n2 - n1) + 17.0 / 3.0) / 2.0
    a4 = ((n1 + n2) + 23.0 / 3.0) / 2.0
    return k * math.exp(lg(a1) - lg(a2) - lg(a3) - lg(a4)) * sg(a1) * sg(a2) * sg(a3) * sg(a4)


@dataclass
class ModeSet:
    modes: np.ndarray        # (M, n, n) float64, scaled by 1/wavelength
    mode_list: list
    tilt_x: int
    tilt_y: int
    atm_rms: np.ndarray      # sqrt(Noll covariance) per mode
    J_T_xy: np.ndarray       # 2x2 tilt Jacobian (alpha -> pixel shift)


def fit_plane(z: np.ndarray, mask: np.ndarray):
    """fitPlane (src/lib/image/utils.cpp:169-233): z = a*y + b*x + c over mask > 0.
    Returns ([a, b, c], chisq/nSamples)."""
    n_y, n_x = z.shape
    yy, xx = np.mgrid[0:n_y, 0:n_x]
    sel = mask.ravel() > 0
    X = np.stack([(yy.ravel() - n_y // 2)[sel], (xx.ravel() - n_x // 2)[sel],
                  np.ones(sel.sum())], axis=1).astype(np.float64)
    d = z.ravel()[sel]
    coef, _, _, _ = np.linalg.lstsq(X, d, rcond=None)
    resid = d - X @ coef
    return coef, float((resid ** 2).sum()) / sel.sum()


def zernike_modeset(mode_list, n_pixels: int, radius: float, wavelength: float,
                    jacobian_scale: float, angle: float = 0.0) -> ModeSet:
    """ModeSet::generate (Zernike) + getNorms/normalize(1/wavelength) + measureJacobian."""
    pupil, _ = make_pupil(n_pixels, radius)
    sup = pupil_support(pupil)
    raw = np.stack([zernike(j, n_pixels, radius, angle) for j in mode_list])
    M = len(mode_list)
    out = np.empty_like(raw)
    for i in range(M):
        nrm = math.sqrt(float((raw[i] * raw[i] * pupil)[pupil > 0].sum()) / sup.area)
        out[i] = raw[i] * ((1.0 / wavelength) / nrm)
    atm = np.array([math.sqrt(zernike_covariance(j, j)) for j in mode_list])
    tx = mode_list.index(2) if 2 in mode_list else -1
    ty = mode_list.index(3) if 3 in mode_list else -1
    J = measure_jacobian(out, pupil, jacobian_scale)
    return ModeSet(out, list(mode_list), tx, ty, atm, J)


@dataclass
class KLMode:
    covariance: float        # eigenvalue of the Zernike covariance block
    weights: list            # [(Noll index, coefficient)]


def kl_expansion(first: int, last: int) -> dict:
    """Zernike::karhunenLoeveExpansion (src/lib/image/zernike.cpp:367-479).

    The Zernike modes first..last are reordered so that modes coupled by the Noll
    covariance form contiguous blocks (the reference's exchange pass); each block's
    covariance matrix is decomposed (singular values in decreasing order, as
    gsl_linalg_SV_decomp returns them); KL mode i takes the singular vector whose column
    is i's position within its block, signed so that its largest coefficient is
    positive.  Returns {i: KLMode}."""
    cov = zernike_covariance
    mapping = {i: i for i in range(first, last + 1)}
    for i in range(first, last):
        cov1 = cov(mapping[i], mapping[last])
        for j in range(last - 1, i, -1):
            cov2 = cov(mapping[i], mapping[j])
            if cov2 == 0.0 and cov1 != 0.0:
                mapping[j], mapping[j + 1] = mapping[j + 1], mapping[j]
            else:
                cov1 = cov2
    reverse = {v: k for k, v in mapping.items()}
    values = {}
    for k in range(first + 1, last + 1):
        values[k] = cov(mapping[k - 1], mapping[k])
    blocks = []
    n = first
    while n <= last:
        b0 = n
        n += 1
        while n <= last and values[n] != 0.0:
            n += 1
        blocks.append((b0, n - 1))
    vectors, singular = {}, {}
    for b0, b1 in blocks:
        size = b1 - b0 + 1
        C = np.array([[cov(mapping[i], mapping[j]) for j in range(b0, b1 + 1)] for i in range(b0, b1 + 1)])
        if size > 1:
            U, S, _ = np.linalg.svd(C)
        else:
            U, S = np.ones((1, 1)), np.array([C[0, 0]])
        vectors[b0] = U
        for k in range(size):
            singular[b0 + k] = float(S[k])
    out = {}
    for i in range(first, last + 1):
        im = reverse[i]
        b0, b1 = next(b for b in blocks if b[0] <= im <= b[1])
        U = vectors[b0]
        col = U[:, im - b0]
        big = int(np.argmax(np.abs(col)))
        sign = -1.0 if col[big] < 0 else 1.0
        out[i] = KLMode(singular[im], [(mapping[b0 + m], sign * float(col[m])) for m in range(b1 - b0 + 1)])
    return out


def kl_modeset(mode_list, n_pixels: int, radius: float, wavelength: float, jacobian_scale: float,
               kl_first: int = 2, kl_last: int = 2000, cutoff: float = 1e-3, angle: float = 0.0) -> ModeSet:
    """ModeSet::generate for Karhunen-Loeve modes (src/lib/momfbd/modes.cpp:158-197, 399-437):
    tilts (Noll 2, 3) stay Zernike; KL mode i is the sum of the normalised Zernike modes
    with |weight| >= cutoff (SVD_REG, default 1e-3), normalised over the pupil; then the same
    getNorms/normalize(1/wavelength) and Jacobian as the Zernike set."""
    pupil, _ = make_pupil(n_pixels, radius)
    sup = pupil_support(pupil)
    kle = kl_expansion(kl_first, kl_last)
    zcache = {}

    def z(j):
        if j not in zcache:
            zcache[j] = zernike(j, n_pixels, radius, angle)
        return zcache[j]

    raw, atm = [], []
    for i in mode_list:
        if i in (2, 3):
            raw.append(z(i))
            atm.append(math.sqrt(zernike_covariance(i, i)))
            continue
        k = kle[i]
        m = np.zeros((n_pixels, n_pixels))
        for j, c in k.weights:
            if abs(c) >= cutoff:
                m += c * z(j)
        nrm = math.sqrt(float(sup.area) / float((m * m * pupil)[pupil > 0].sum()))
        raw.append(m * nrm)
        atm.append(math.sqrt(k.covariance))
    raw = np.stack(raw)
    out = np.empty_like(raw)
    for i in range(raw.shape[0]):
        nrm = math.sqrt(float((raw[i] * raw[i] * pupil)[pupil > 0].sum()) / sup.area)
        out[i] = raw[i] * ((1.0 / wavelength) / nrm)
    tx = list(mode_list).index(2) if 2 in mode_list else -1
    ty = list(mode_list).index(3) if 3 in mode_list else -1
    J = measure_jacobian(out, pupil, jacobian_scale)
    return ModeSet(out, list(mode_list), tx, ty, np.array(atm), J)


def measure_jacobian(modes: np.ndarray, pupil: np.ndarray, scale: float) -> np.ndarray:
    """ModeSet::measureJacobian (src/lib/momfbd/modes.cpp:464-512); returns J_T_xy."""
    fits = []
    for i in range(modes.shape[0]):
        c, chisq = fit_plane(modes[i], pupil)
        fits.append(((chisq, c[0], c[1], c[2]), i))
    fits.sort()
    J = np.zeros((2, 2))
    chis = [fits[k][0][0] for k in range(min(3, len(fits)))]
    for cnt in range(2):
        key = fits[cnt][0]
        J[0, cnt] = scale * key[2]
        J[1, cnt] = scale * key[1]
    if len(chis) > 2 and 100 * chis[0] < chis[2] and 100 * chis[1] < chis[2]:
        if abs(J[0, 0]) / abs(J[1, 0]) < 1:
            J[:, [0, 1]] = J[:, [1, 0]]
    return J


def apodize_window(size: int, blend: int) -> np.ndarray:
    """apodizeInPlace(window, blend) on an all-ones array (src/lib/image/utils.cpp:584-614)."""
    w = np.ones((size, size))
    if blend <= 0:
        return w
    b = min(blend, size // 2)
    tmp = np.zeros(b + 2)
    nn = b + 2
    step = math.pi / (nn - 1)
    for i in range(1, nn):
        tmp[i] = 0.5 + (-0.5) * math.cos(i * step)     # math::apodize(tmp, n, 1.0), tmp[0] = 0
    for r in range(b):
        w[r, :] *= tmp[r + 1]
        w[size - r - 1, :] *= tmp[r + 1]
    for c in range(b):
        w[:, c] *= tmp[c + 1]
        w[:, size - c - 1] *= tmp[c + 1]
    return w


def solver_windows(patch_size: int, apodization: int = -1):
    """Solver::init window and noiseWindow (src/lib/momfbd/solver.cpp:113-126)."""
    apod = patch_size // 8 if apodization < 0 else apodization
    if apod:
        return apodize_window(patch_size, apod), apodize_window(patch_size, apod // 2)
    return np.ones((patch_size, patch_size)), np.ones((patch_size, patch_size))


@dataclass
class NullSpace:
    n_parameters: int
    n_free: int
    rows: np.ndarray   # int32 parameter index (image * M + mode)
    cols: np.ndarray   # int32 free-parameter index
    vals: np.ndarray   # float64

    def dense(self) -> np.ndarray:
        A = np.zeros((self.n_parameters, self.n_free))
        np.add.at(A, (self.rows, self.cols), self.vals)
        return A


def build_constraints(image_wavefronts, n_modes: int, ref_images, tilt_modes=(0, 1)) -> NullSpace:
    """Null-space map of the MOMFBD linear constraints.

    The constraints are those of Constraints::init (src/lib/momfbd/constraints.cpp:536-622):
    for every mode, images that share a wavefront share the coefficient; for the two
    tilt modes (mode indices 0 and 1) the coefficients of the first object's first
    channel (``ref_images``) also sum to zero.

    The reference builds an orthonormal basis of the null space group by group
    (constraints.cpp:85-198, 429-469).  The solver only uses the map through
    alpha = offset + N beta and grad_beta = N^T grad_alpha, and its conjugate-gradient
    iteration only forms norms and dot products of beta-space vectors; for any two
    orthonormal bases N and N R (R orthogonal) those are equal, so the alpha-space
    trajectory does not depend on which orthonormal basis is used.  This builder
    therefore uses the simplest sparse orthonormal basis of the same null space:
    one 1/sqrt(k) column per shared wavefront for non-tilt modes, and an orthonormal
    basis of the zero-sum subspace over wavefronts for the tilt modes.
    """
    I = len(image_wavefronts)
    wf = np.asarray(image_wavefronts)
    groups = {}
    for j, w in enumerate(wf):
        groups.setdefault(int(w), []).append(j)
    order = sorted(groups.keys(), key=lambda w: groups[w][0])
    ref = set(int(r) for r in ref_images)
    rows, cols, vals = [], [], []
    col = 0
    for m in range(n_modes):
        if m in tilt_modes:
            # u_g = sqrt(|g|) t_g;  constraint  sum_g n_ref(g)/sqrt(|g|) u_g = 0
            c = np.array([sum(1 for j in groups[w] if j in ref) / math.sqrt(len(groups[w]))
                          for w in order])
            G = len(order)
            if np.any(c != 0):
                # orthonormal basis of the complement of c (Householder reflection)
                v = c / np.linalg.norm(c)
                e = np.zeros(G); e[0] = 1.0
                h = v - e
                if np.linalg.norm(h) < 1e-14:
                    H = np.eye(G)
                else:
                    h /= np.linalg.norm(h)
                    H = np.eye(G) - 2.0 * np.outer(h, h)
                basis = H[:, 1:]          # columns orthogonal to v
            else:
                basis = np.eye(G)
            for k in range(basis.shape[1]):
                for gi, w in enumerate(order):
                    val = basis[gi, k] / math.sqrt(len(groups[w]))
                    if abs(val) > 1e-10:
                        for j in groups[w]:
                            rows.append(j * n_modes + m); cols.append(col); vals.append(val)
                col += 1
        else:
            for w in order:
                g = groups[w]
                val = 1.0 / math.sqrt(len(g))
                for j in g:
                    rows.append(j * n_modes + m); cols.append(col); vals.append(val)
                col += 1
    return NullSpace(I * n_modes, col, np.array(rows, np.int32), np.array(cols, np.int32),
                     np.array(vals, np.float64))


def reg_alpha_weights(atm_rms, n_images: int, patch_size: int, wavelength: float, reg_alpha: float):
    """Solver::regAlphaWeights (solver.cpp:147-156): for every image and mode
    reg_alpha / wavelength * nTotalPixels / atm_rms[m]^2 (0 where atm_rms is 0), nTotalPixels =
    images * patch_size^2; the metric gains 0.5 sum alpha^2 w.  Returns [n_images][M]."""
    rms = np.asarray(atm_rms, np.float64)
    scale = reg_alpha / wavelength * (n_images * patch_size * patch_size)
    w = np.where(rms == 0.0, 0.0, scale / np.where(rms == 0.0, 1.0, rms * rms))
    return np.tile(w, (n_images, 1))
