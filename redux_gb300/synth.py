"""Seeded synthetic MOMFBD workloads.

No SST data is available, so every workload is synthetic: an object field (Gaussian
random field with a k^-2 power spectrum, mean 1, 10 % RMS contrast), per-frame
Kolmogorov wavefronts expanded in Zernike modes, images = object (x) PSF with
Poisson noise at 1e4 photons/px plus N(0, 10^2) read noise, stored as float32.

The named workloads (`workload`): "plain64", one 64 x 64 patch, 2 channels x 4 frames,
Zernike modes Noll 2..21; "adjoint88", 88 x 88, 3 channels x 8 frames, 36 Karhunen-Loeve
modes; "production88", 225 patches 88 x 88, 3 channels x 12 frames, 36 KL modes;
"large128", 256 patches 128 x 128, 3 channels x 32 frames, 100 KL modes.  KL modes keep the
tilts Zernike and come from the expansion of the Noll covariance.  The uneven batch
(`uneven_batch`: sizes {64, 88, 128}, 8-24 frames, 36-60 modes) is a list of workloads,
one per patch geometry.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.fft as sfft

from . import jobsetup as js

WAVELENGTH = 630.2e-9
TELESCOPE_D = 0.97
ARCSEC_PER_PX = WAVELENGTH / (2.0 * TELESCOPE_D) / js.RADIANS_PER_ARCSEC   # critical sampling
MAX_LOCAL_SHIFT = 5


@dataclass
class Job:
    """Static (per job) inputs of the per-patch solver."""
    otf_size: int
    pupil_pixels: int
    patch_size: int
    n_modes: int
    modes: np.ndarray            # (M, n, n) float64, scaled by 1/lambda
    mode_list: list
    tilt_x: int
    tilt_y: int
    J_T_xy: np.ndarray
    pupil: np.ndarray            # (n, n)
    support: js.PupilSupport
    img_object: np.ndarray       # (I,) int32
    img_channel: np.ndarray      # (I,) int32, global channel index
    img_wavefront: np.ndarray    # (I,) int32
    phi_fixed: np.ndarray        # (C, n, n) float64, diversity phase per channel
    obj_weight: np.ndarray       # (nObj,)
    obj_grad_step: np.ndarray    # (nObj,) GRADDIFF_STEP * wavelength
    window: np.ndarray           # (ps, ps)
    noise_window: np.ndarray     # (ps, ps)
    nullspace: js.NullSpace
    cutout_size: int
    channel_div_pv: np.ndarray   # (C,) diversity defocus of each channel, waves PV
    wavelength: float = WAVELENGTH
    basis: str = "zernike"       # "zernike" or "kl"
    atm_var: np.ndarray = None   # (M,) Kolmogorov variance of each mode at D/r0 = 1
    kl_weights: dict = None      # KL mode -> [(Noll index, weight)] (basis "kl")
    kl_cutoff: float = 1e-3

    @property
    def n_images(self):
        return int(self.img_object.shape[0])

    @property
    def n_objects(self):
        return int(self.obj_weight.shape[0])

    @property
    def n_channels(self):
        return int(self.phi_fixed.shape[0])


@dataclass
class Patches:
    cutouts: np.ndarray          # (P, I, cs, cs) float32
    residual_alpha: np.ndarray   # (P, I, 2) float64 (y, x)
    fixed_gamma: np.ndarray | None  # (P, nObj) or None (noise-derived)
    alpha_true: np.ndarray       # (P, I, M) float64 (reference units, lambda * rad)


@dataclass
class Workload:
    name: str
    job: Job
    patches: Patches
    cfg: dict = field(default_factory=dict)


def _grf(rng, size, contrast=0.1):
    """Gaussian random field with power ~ k^-2, mean 1 and RMS contrast `contrast`."""
    w = rng.standard_normal((size, size))
    f = np.fft.fft2(w)
    ky = np.fft.fftfreq(size)[:, None]
    kx = np.fft.fftfreq(size)[None, :]
    k = np.sqrt(kx * kx + ky * ky)
    amp = np.zeros_like(k)
    amp[k > 0] = 1.0 / k[k > 0]
    g = np.real(np.fft.ifft2(f * amp))
    g -= g.mean()
    g *= contrast / g.std()
    return 1.0 + g


_PUPILS = {}


def _pupil_cached(n, radius):
    key = (n, radius)
    if key not in _PUPILS:
        _PUPILS[key] = js.make_pupil(n, radius)[0]
    return _PUPILS[key]


_ZCACHE = {}


def _zernike_cached(j, n, radius):
    key = (j, n, radius)
    z = _ZCACHE.get(key)
    if z is None:
        z = js.zernike(j, n, radius)
        _ZCACHE[key] = z
    return z


def make_job(N: int, n_modes: int, layout, grad_step=1e-2, apodization=-1, basis="zernike",
             kl_last=None) -> Job:
    """layout: list of objects, each a list of channels (diversity PV waves), and the
    number of frames; e.g. [[0.0, 1.0]] = one object with a focus and a +1 wave channel.
    basis "kl": Karhunen-Loeve modes 2..n_modes+1 (tilts Zernike) from the expansion over
    Noll 2..kl_last (default 2 * n_modes + 1, KL_MAX_MODE >= 2 M)."""
    frames = layout["frames"]
    objects = layout["objects"]
    fc, radius, npup = js.calculate_pupil_size(N, WAVELENGTH, TELESCOPE_D, ARCSEC_PER_PX)
    assert npup * 2 == 2 * (N // 2) and 2 * npup == 2 * npup
    n = npup
    otf = 2 * n
    mode_list = list(range(2, 2 + n_modes))
    jscale = WAVELENGTH * (0.5 * fc) / ((math.pi * math.pi / 648000.0) * ARCSEC_PER_PX * TELESCOPE_D)
    kl = None
    if basis == "kl":
        kl_last = kl_last or 2 * n_modes + 1
        ms = js.kl_modeset(mode_list, n, radius, WAVELENGTH, jscale, 2, kl_last)
        kl = {i: e.weights for i, e in js.kl_expansion(2, kl_last).items() if i in mode_list}
    else:
        ms = js.zernike_modeset(mode_list, n, radius, WAVELENGTH, jscale)
    pupil, _ = js.make_pupil(n, radius)
    sup = js.pupil_support(pupil)
    img_obj, img_ch, img_wf, phis, ref = [], [], [], [], []
    ch_index = 0
    z4 = js.zernike(4, n, radius)
    for o, chans in enumerate(objects):
        for c, pv_waves in enumerate(chans):
            phis.append((math.pi / math.sqrt(3.0)) * pv_waves * z4)
            for t in range(frames):
                if o == 0 and c == 0:
                    ref.append(len(img_obj))
                img_obj.append(o); img_ch.append(ch_index); img_wf.append(t)
            ch_index += 1
    win, nwin = js.solver_windows(N, apodization)
    ns = js.build_constraints(img_wf, n_modes, ref)
    return Job(otf_size=otf, pupil_pixels=n, patch_size=N, n_modes=n_modes, modes=ms.modes,
               mode_list=mode_list, tilt_x=ms.tilt_x, tilt_y=ms.tilt_y, J_T_xy=ms.J_T_xy,
               pupil=pupil, support=sup,
               img_object=np.array(img_obj, np.int32), img_channel=np.array(img_ch, np.int32),
               img_wavefront=np.array(img_wf, np.int32), phi_fixed=np.stack(phis),
               obj_weight=np.ones(len(objects)), obj_grad_step=np.full(len(objects), grad_step * WAVELENGTH),
               window=win, noise_window=nwin, nullspace=ns, cutout_size=N + 2 * MAX_LOCAL_SHIFT,
               channel_div_pv=np.array([pv for chans in objects for pv in chans]),
               basis=basis, atm_var=np.asarray(ms.atm_rms) ** 2, kl_weights=kl)


def _basis_cached(job: Job, n, radius):
    """The job's modes at unit RMS on an n x n generator pupil (Zernike or KL combinations,
    normalised over that pupil as ModeSet normalises them)."""
    zs = []
    for i in job.mode_list:
        if job.basis != "kl" or i in (2, 3):
            zs.append(_zernike_cached(i, n, radius))
            continue
        m = np.zeros((n, n))
        for j, c in job.kl_weights[i]:
            if abs(c) >= job.kl_cutoff:
                m += c * _zernike_cached(j, n, radius)
        pupil = _pupil_cached(n, radius)
        m *= math.sqrt(float(pupil.sum()) / float((m * m * pupil)[pupil > 0].sum()))
        zs.append(m)
    return np.stack(zs)


def make_patches(job: Job, n_patches: int, d_r0: float, rng, fixed_gamma=None,
                 photons=1e4, read_noise=10.0, K=None, tilt_scale=1.0) -> Patches:
    """Images of `n_patches` independent patches (one object field per object and patch)."""
    N, cs = job.patch_size, job.cutout_size
    I, M = job.n_images, job.n_modes
    frames = int(job.img_wavefront.max()) + 1
    if K is None:
        K = 1 << int(math.ceil(math.log2(cs + 64)))
    var = np.asarray(job.atm_var) * d_r0 ** (5.0 / 3.0)
    sd = np.sqrt(var)
    n_obj = job.n_objects
    cut = np.zeros((n_patches, I, cs, cs), np.float32)
    alpha = np.zeros((n_patches, I, M))
    n = K // 2
    radius = n / 2.0
    pupil = _pupil_cached(n, radius)
    Zk = _basis_cached(job, n, radius)
    z4 = _zernike_cached(4, n, radius)
    o0 = (K - cs) // 2
    op = (K - n) // 2
    for p in range(n_patches):
        a_wf = rng.standard_normal((frames, M)) * sd
        for tm in (job.tilt_x, job.tilt_y):
            if tm >= 0:
                a_wf[:, tm] *= tilt_scale
        # tilts of the reference channel sum to zero (the constraint the solver imposes)
        for tm in (job.tilt_x, job.tilt_y):
            if tm >= 0:
                a_wf[:, tm] -= a_wf[:, tm].mean()
        objs = [_grf(rng, K) for _ in range(n_obj)]
        objs_ft = np.stack([sfft.fft2(o, workers=-1) for o in objs])
        # all images of the patch at once: phase on a K/2 pupil, PSF = |ifft(P)|^2 (the
        # solver's convention, S = c^2 ifft(|fft(P)|^2)), circular convolution on K x K
        phase = np.tensordot(a_wf, Zk, 1)                     # (frames, n, n)
        pf = np.zeros((I, K, K), np.complex64)
        for j in range(I):
            c = int(job.img_channel[j]); t = int(job.img_wavefront[j])
            ph = phase[t] + float(job.channel_div_pv[c]) * (math.pi / math.sqrt(3.0)) * z4
            pf[j, op:op + n, op:op + n] = (pupil * np.exp(1j * ph)).astype(np.complex64)
        psf = np.abs(sfft.ifft2(pf, axes=(-2, -1), workers=-1)) ** 2
        psf /= psf.sum(axis=(-2, -1), keepdims=True)
        otf = sfft.fft2(psf, axes=(-2, -1), workers=-1)
        img = np.real(sfft.ifft2(objs_ft[job.img_object].astype(np.complex64) * otf, axes=(-2, -1), workers=-1))
        reg = np.clip(img[:, o0:o0 + cs, o0:o0 + cs], 0, None) * photons
        noisy = rng.poisson(reg).astype(np.float64) + rng.normal(0.0, read_noise, reg.shape)
        cut[p] = noisy.astype(np.float32)
        for j in range(I):
            alpha[p, j] = a_wf[int(job.img_wavefront[j])] * job.wavelength
    fg = None
    if fixed_gamma is not None:
        fg = np.full((n_patches, n_obj), float(fixed_gamma))
    return Patches(cutouts=cut, residual_alpha=np.zeros((n_patches, I, 2)), fixed_gamma=fg,
                   alpha_true=alpha)


LAYOUT_1OBJ = lambda frames: {"frames": frames, "objects": [[0.0, 1.0]]}          # focus + diversity
LAYOUT_WB_NB = lambda frames: {"frames": frames, "objects": [[0.0], [0.0, 1.0]]}  # WB; NB focus + div


UNEVEN_SIZES = (64, 88, 128)
UNEVEN_KL_LAST = 121   # one expansion over Noll 2..121 for every mode count (its first M modes)


def uneven_batch(n_patches: int = 400, frames=(8, 24), modes=(36, 60), levels: int | None = None,
                 d_r0: float = 15.0, seed_offset: int = 0) -> list:
    """The uneven batch: patches whose size ({64, 88, 128}), frames per channel (8..24) and
    number of KL modes (36..60) are drawn uniformly per patch, 3 channels (wideband; narrowband
    focus and +1 wave), grouped by geometry.  levels: draw frames and modes from that many
    evenly spaced values instead (e.g. 3: frames {8, 16, 24}, modes {36, 48, 60}) so that
    patches share geometries.  Returns one Workload per distinct (size, frames, modes), its
    cfg["patch_index"] the positions of its patches in the draw order."""
    rng = np.random.default_rng(20261203 + WORKLOAD_SEEDS["uneven"] + seed_offset)

    def draw(lo, hi):
        if levels:
            return int(np.linspace(lo, hi, levels).round().astype(int)[rng.integers(levels)])
        return int(rng.integers(lo, hi + 1))

    draws = [(int(UNEVEN_SIZES[rng.integers(len(UNEVEN_SIZES))]), draw(*frames), draw(*modes))
             for _ in range(n_patches)]
    groups = {}
    for i, g in enumerate(draws):
        groups.setdefault(g, []).append(i)
    out = []
    for (N, F, M), idx in sorted(groups.items()):
        job = make_job(N, M, LAYOUT_WB_NB(F), basis="kl", kl_last=UNEVEN_KL_LAST)
        prng = np.random.default_rng([20261203 + WORKLOAD_SEEDS["uneven"] + seed_offset, N, F, M])
        pt = make_patches(job, len(idx), d_r0, prng)
        out.append(Workload(f"uneven {N}x{N}, 3ch x {F}fr, {M} KL modes", job, pt, dict(patch_index=idx)))
    return out


# seed of each named workload: 20261203 + this (+ seed_offset)
WORKLOAD_SEEDS = {"plain64": 0, "adjoint88": 1, "production88": 2, "uneven": 3, "large128": 4}


def workload(name: str, n_patches: int | None = None, seed_offset: int = 0, frames=None) -> Workload:
    """A named benchmark workload (module docstring), seeded with 20261203 + its
    WORKLOAD_SEEDS entry (+ seed_offset); n_patches and frames override its sizes."""
    if name not in WORKLOAD_SEEDS or name == "uneven":
        raise ValueError(f"unknown workload {name!r} (the uneven batch comes from uneven_batch)")
    rng = np.random.default_rng(20261203 + WORKLOAD_SEEDS[name] + seed_offset)
    if name == "plain64":
        job = make_job(64, 20, LAYOUT_1OBJ(frames or 4))
        pt = make_patches(job, n_patches or 1, 10.0, rng, fixed_gamma=1e-3)
        cfg = dict(iterations=50, gamma=1e-3)
        return Workload("plain FP64 64x64, 2ch x 4fr, Z2-21", job, pt, cfg)
    if name == "adjoint88":
        job = make_job(88, 36, LAYOUT_WB_NB(frames or 8), basis="kl")
        pt = make_patches(job, n_patches or 1, 10.0, rng)
        return Workload("adjoint check 88x88, 3ch x 8fr, 36 modes", job, pt, {})
    if name == "production88":
        job = make_job(88, 36, LAYOUT_WB_NB(frames or 12), basis="kl")
        pt = make_patches(job, n_patches or 225, 15.0, rng)
        return Workload("production 88x88, 3ch x 12fr, 36 KL modes", job, pt, dict(iterations=100))
    job = make_job(128, 100, LAYOUT_WB_NB(frames or 32), basis="kl")
    pt = make_patches(job, n_patches or 256, 25.0, rng)
    return Workload("mixed precision 128x128, 3ch x 32fr, 100 KL modes", job, pt, {})
