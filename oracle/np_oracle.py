"""Independent numpy FP64 restatement of the per-image model (test infrastructure).

Written directly from the reference's formulas, with numpy's FFT instead of the oracle's
own, to cross-check oracle.c:
  OTF  S = fftshift(ifft(|fft(c PF embedded at n/2)|^2))     subimage.cpp:586-612
  P = sum_j conj(D_j) S_j,  Q = gamma + sum_j |S_j|^2          subimage.cpp:226-234
  L = sum_obj w sum_support (sum_j |D_j|^2 - |P|^2/Q) / ps^2   object.cpp:597-615
  Vogel gradient, literally as calcVogelWeight/gradientVogel   subimage.cpp:312-390
  exact gradient  dL/dphi = -4 c^2 / ps^2 Im(conj(PF) (G * PF))
"""
from __future__ import annotations

import numpy as np


class NumpyModel:
    def __init__(self, job, D, gamma, otf_norm):
        self.job = job
        self.D = D                      # (I, N, N) centred image transforms
        self.gamma = np.asarray(gamma)  # (nObj,)
        self.c = np.asarray(otf_norm)   # (C,)
        N = job.otf_size
        m = np.zeros(N * N, bool)
        m[job.support.otf_support] = True
        self.mask = m.reshape(N, N)

    def phase(self, alpha):
        j = self.job
        return j.phi_fixed[j.img_channel] + np.tensordot(alpha, j.modes, axes=([1], [0]))

    def otf(self, alpha):
        j = self.job
        N, n = j.otf_size, j.pupil_pixels
        phi = self.phase(alpha)
        PF = j.pupil[None] * np.exp(1j * phi)
        big = np.zeros((j.n_images, N, N), complex)
        big[:, n // 2:n // 2 + n, n // 2:n // 2 + n] = PF * self.c[j.img_channel][:, None, None]
        X = np.fft.fft2(big)
        S = np.fft.fftshift(np.fft.ifft2(np.abs(X) ** 2), axes=(-2, -1))
        return S, PF

    def pq(self, S):
        j = self.job
        P = np.zeros((j.n_objects,) + S.shape[1:], complex)
        Q = np.zeros((j.n_objects,) + S.shape[1:]) + self.gamma[:, None, None]
        F = np.zeros_like(Q)
        for i in range(j.n_images):
            o = j.img_object[i]
            P[o] += np.conj(self.D[i]) * S[i]
            Q[o] += np.abs(S[i]) ** 2
            F[o] += np.abs(self.D[i]) ** 2
        return P, Q, F

    def metric(self, alpha):
        j = self.job
        S, _ = self.otf(alpha)
        P, Q, F = self.pq(S)
        L = 0.0
        for o in range(j.n_objects):
            t = (F[o] - np.abs(P[o]) ** 2 / Q[o])[self.mask].sum() / j.patch_size ** 2
            L += j.obj_weight[o] * t
        return L

    def gradient(self, alpha, kind="vogel"):
        j = self.job
        N, n, M = j.otf_size, j.pupil_pixels, j.n_modes
        S, PF = self.otf(alpha)
        P, Q, _ = self.pq(S)
        A = j.pupil
        area = float(A.ravel()[j.support.pupil_support].sum())
        g = np.zeros((j.n_images, M))
        for i in range(j.n_images):
            o = j.img_object[i]
            G = (P[o] * Q[o] * self.D[i] - np.abs(P[o]) ** 2 * S[i]) / Q[o] ** 2 * self.mask
            p = np.zeros((N, N), complex)
            p[:n, :n] = PF[i]
            conv = np.fft.ifft2(np.fft.fft2(np.fft.ifftshift(G)) * np.fft.fft2(p))[:n, :n]   # (G * PF)
            w = j.obj_weight[o]
            if kind == "vogel":
                v = np.imag(np.conj(PF[i]) * conv) * A / N ** 2
                g[i] = (-2.0 * area / N ** 2) * w * w * np.tensordot(j.modes, v, 2)
            else:
                c = self.c[j.img_channel[i]]
                dphi = -(4.0 * c * c / j.patch_size ** 2) * np.imag(np.conj(PF[i]) * conv) * (A > 0)
                g[i] = w * np.tensordot(j.modes, dphi, 2)
        return g


# ---------------------------------------------------------------------------------------
# Restoration (Object::restorePatch, object.cpp:278-334; ScharmerFilter, smooth,
# connectedRegion in image/utils.cpp:49-57, 295-392), an independent numpy statement used
# to cross-check the C restatement.
# ---------------------------------------------------------------------------------------
def smooth(d, nY, nX):
    """Mean over the clipped window [y-nY, y+nY) x [x-nX, x+nX) (upper bounds exclusive)."""
    ny, nx = d.shape
    ii = np.zeros((ny + 1, nx + 1))
    ii[1:, 1:] = np.cumsum(np.cumsum(d, 0), 1)
    y = np.arange(ny)[:, None]
    x = np.arange(nx)[None, :]
    yl, yh = np.maximum(y - nY, 0), np.minimum(y + nY, ny)
    xl, xh = np.maximum(x - nX, 0), np.minimum(x + nX, nx)
    tot = ii[yh, xh] - ii[yl, xh] - ii[yh, xl] + ii[yl, xl]
    return tot / ((yh - yl) * (xh - xl))


def scharmer_filter(data, q2, noise_power, frequency_cutoff):
    from scipy import ndimage
    N = data.shape[0]
    with np.errstate(divide="ignore"):
        pt = (noise_power * N * N) / smooth(np.abs(data) ** 2 * q2, 1, 1)
    mirror = pt[(-np.arange(N)) % N][:, (-np.arange(N)) % N]
    rr = np.maximum(1.0 - 0.5 * (mirror + pt), 0.0)
    rr[rr < 0.2] = 0.0
    rr[rr > 1.0] = 1.0
    rr[N // 2, N // 2] = 1.0
    lab, _ = ndimage.label(rr > 0.0, structure=[[0, 1, 0], [1, 1, 1], [0, 1, 0]])
    rr = rr * (lab == lab[N // 2, N // 2])
    rr = smooth(rr, 4, 4)
    y, x = np.mgrid[0:N, 0:N]
    out = data * rr
    out[(y - N // 2) ** 2 + (x - N // 2) ** 2 > frequency_cutoff ** 2] = 0.0
    return out


def restore(D, S, noise, image_object, obj, frequency_cutoff, ps, support, no_filter=False):
    """Restored object obj from centred image transforms D and OTFs S [I][N][N]; sums over
    the OTF support (flat centred indices) only, as SubImage::restore."""
    idx = [j for j in range(len(image_object)) if image_object[j] == obj]
    mask = np.zeros(D[0].size, bool)
    mask[np.asarray(support)] = True
    mask = mask.reshape(D[0].shape)
    num = sum(np.conj(D[j]) * S[j] for j in idx) * mask
    den = sum(np.abs(S[j]) ** 2 for j in idx) * mask
    nv = float(np.mean([noise[j] ** 2 for j in idx]))
    O = np.where(den != 0.0, np.conj(num) / np.where(den != 0.0, den, 1.0), 0.0)
    if not no_filter:
        O = scharmer_filter(O, den, nv, 0.9 * frequency_cutoff)
    N = O.shape[0]
    img = np.real(np.fft.ifft2(np.fft.ifftshift(O)))
    off = (N - ps) // 2
    return img[off:off + ps, off:off + ps]


def restore_outputs(D, S, image_object, objects, ps):
    """The other outputs of Object::restorePatch (object.cpp:335-383) from centred image
    transforms D and OTFs S [I][N][N] and the untrimmed float objects [nObj][N][N]:
      PSF_j  = reorder(real(ift(reorder(S_j))) / N^2)   SubImage::addPSF (subimage.cpp:615-626)
               with the OTF's flags REORDER_IMG|REORDER_FT|NORMALIZE_FT, centred (89-90)
      mean   = float(float(sum_j PSF_j) / count)         object.cpp:345-350
      cobj_j = real(ift(ft(img_o) / N^2 * reorder(S_j)))  FourierTransform::convolve
               (fouriertransform.hpp:310-324): image not reordered, product un-centred
      res_j  = float(float(cobj_j) - real(ift(reorder(D_j))) / N^2)   subimage.hpp:118-129
    All trimmed to ps around the centre.  Returns (psf [I], psf_mean [nObj], cobj [I], res [I])."""
    I, N = S.shape[0], S.shape[1]
    off = (N - ps) // 2
    cut = (slice(off, off + ps), slice(off, off + ps))
    psf = np.array([np.fft.fftshift(np.real(np.fft.ifft2(np.fft.ifftshift(S[j])))) for j in range(I)])
    nObj = len(objects)
    psf_mean = []
    for o in range(nObj):
        idx = [j for j in range(I) if image_object[j] == o]
        acc = np.zeros((N, N))
        for j in idx:
            acc += psf[j]
        psf_mean.append((acc.astype(np.float32).astype(np.float64) * (1.0 / len(idx))).astype(np.float32)[cut])
    F = [np.fft.fft2(np.asarray(objects[o], np.float32).astype(np.float64)) for o in range(nObj)]
    cobj = np.array([np.real(np.fft.ifft2(F[image_object[j]] * np.fft.ifftshift(S[j]))) for j in range(I)])
    img = np.array([np.real(np.fft.ifft2(np.fft.ifftshift(D[j]))) for j in range(I)])
    res = (cobj.astype(np.float32).astype(np.float64) - img).astype(np.float32)
    return (psf.astype(np.float32)[:, cut[0], cut[1]], np.array(psf_mean),
            cobj.astype(np.float32)[:, cut[0], cut[1]], res[:, cut[0], cut[1]])
