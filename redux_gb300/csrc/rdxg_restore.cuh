// Restoration of the objects of every patch: Object::restorePatch (object.cpp:278-334) for
// the restored object, with SubImage::restore (subimage.cpp:242-256) and ScharmerFilter,
// smooth and connectedRegion (image/utils.cpp:49-57, 295-392).  FP64 throughout (the image
// transforms and OTFs enter as stored, FP32 or FP64): one block per (patch, object), the
// N x N work arrays in global scratch, the final inverse transform in shared memory.
#pragma once

#include "rdxg_kernels.cuh"

namespace rdxg {

struct RestoreArgs {
    const double* fc;      // [nObj] Object::frequencyCutoff (the filter uses 0.9 of it)
    int32_t noFilter;      // RF_NO_FILTER
    double* scratch;       // [P * nObj][kRestoreScratch * N * N]
    float* out;            // [P][nObj][ps][ps]
    float* objFull;        // [P][nObj][N][N] the untrimmed float object (ObjectData::img before trim), or null
};

// Optional outputs of Object::restorePatch (object.cpp:335-383): PSFs, convolved objects and
// residuals, trimmed to the patch like the object.
enum : int32_t { kRestorePsf = 1, kRestorePsfAvg = 2, kRestoreCobj = 4, kRestoreResidual = 8 };
struct RestoreOutArgs {
    int32_t flags;
    const float* objFull;  // [P][nObj][N][N]
    cx<double>* Fo;        // [P][nObj][N][N] unnormalised transform of the float object
    double* pool;          // [blocks][3 * N * N] per-block work: W (complex N x N) + one real N x N
    float* psf;            // [P][I][ps][ps] (kRestorePsf) or [P][nObj][ps][ps] (kRestorePsfAvg)
    float* cobj;           // [P][I][ps][ps]
    float* res;            // [P][I][ps][ps]
};
constexpr int kRestoreScratch = 7;   // doubles per frequency: object (2), den, pt, rr, tmp, mask
constexpr int kRestoreBand = 16;     // lines per band of the banded transforms (at most)
// lines per band for an N x N transform: a divisor of N (16, or 8 for N = 88)
template <int N> struct Band { static constexpr int value = N % kRestoreBand == 0 ? kRestoreBand : 8; };

// 2-D transform (DIR -1 forward, +1 backward, unnormalised) of the N x N array given by
// load(y, x), in bands of Band<N> lines through shared memory s ([B][LDS]) with the row
// results in W (N x N, global); store(y, x, v) receives every output value once.
template <int N, int DIR, int THREADS, typename Load, typename Store>
__device__ __forceinline__ void fft2_banded(Load load, Store store, cx<double>* W, cx<double>* s,
                                            const cx<double>* tw) {
    constexpr int B = Band<N>::value, LDS = Tile<N>::LDS;
    static_assert(N % B == 0, "bands tile the array");
    for (int r0 = 0; r0 < N; r0 += B) {
        __syncthreads();
        for (int i = threadIdx.x; i < B * N; i += THREADS) s[(i / N) * LDS + i % N] = load(r0 + i / N, i % N);
        __syncthreads();
        fft_lines<double, N, DIR, B, true, THREADS>(s, 0, tw, threadIdx.x);
        for (int i = threadIdx.x; i < B * N; i += THREADS) W[(r0 + i / N) * N + i % N] = s[(i / N) * LDS + i % N];
    }
    for (int c0 = 0; c0 < N; c0 += B) {
        __syncthreads();
        for (int i = threadIdx.x; i < B * N; i += THREADS) {
            const int col = c0 + i % B, y = i / B;
            s[(i % B) * LDS + y] = W[y * N + col];
        }
        __syncthreads();
        fft_lines<double, N, DIR, B, true, THREADS>(s, 0, tw, threadIdx.x);
        for (int i = threadIdx.x; i < B * N; i += THREADS) store(i % N, c0 + i / N, s[(i / N) * LDS + i % N]);
    }
    __syncthreads();
}

template <int N, int THREADS>
__device__ __forceinline__ void restore_twiddles(cx<double>* tw) {
    for (int k = threadIdx.x; k < N; k += THREADS) {
        double sn, cs;
        sincospi(2.0 * k / N, &sn, &cs);
        tw[k] = mkc<double>(cs, -sn);
    }
}

// smooth (utils.cpp:304-328): mean over [y-nY, y+nY) x [x-nX, x+nX) clipped to the array, the
// sum in the reference's order
template <int N, int THREADS>
__device__ __forceinline__ void restore_smooth(const double* in, double* out, int nY, int nX) {
    for (int c = threadIdx.x; c < N * N; c += THREADS) {
        const int y = c / N, x = c % N;
        const int yl = max(y - nY, 0), yh = min(y + nY, N), xl = max(x - nX, 0), xh = min(x + nX, N);
        double t = 0;
        int cnt = 0;
        for (int yy = yl; yy < yh; ++yy)
            for (int xx = xl; xx < xh; ++xx) { t += in[yy * N + xx]; cnt++; }
        out[c] = t / cnt;
    }
    __syncthreads();
}

template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_restore(KParams<T> kp, RestoreArgs ra) {
    constexpr int N2 = N * N, LDS = Tile<N>::LDS;
    const int b = blockIdx.x;
    const int p = b / kp.nObj, o = b % kp.nObj;
    double* sc = ra.scratch + (size_t)b * kRestoreScratch * N2;
    double2* obj = reinterpret_cast<double2*>(sc);
    double* den = sc + 2 * N2;
    double* pt = den + N2;
    double* rr = pt + N2;
    double* tmp = rr + N2;
    int* mask = reinterpret_cast<int*>(tmp + N2);
    __shared__ double noiseVar;
    __shared__ int changed;
    const int first = kp.pObjFirst[(size_t)p * kp.nObj + o], cnt = kp.pObjCount[(size_t)p * kp.nObj + o];
    const size_t g0 = (size_t)p * kp.I + first;
    // sum_j conj(D_j) S_j and sum_j |S_j|^2 on the support, images in order; conjugate;
    // Array::safeDivide (eps = 0)
    for (int c = threadIdx.x; c < N2; c += THREADS) {
        double2 num = make_double2(0, 0);
        double d = 0;
        if (kp.otfMask[c]) {
            for (int j = 0; j < cnt; ++j) {
                const cx<T> Dv = kp.D[(g0 + j) * N2 + c];
                const cx<T> S = kp.S[(g0 + j) * N2 + c];
                const double dr = Dv.x, di = Dv.y, sr = S.x, si = S.y;
                d += sr * sr + si * si;
                num.x += dr * sr + di * si;   // conj(D) S
                num.y += dr * si - di * sr;
            }
        }
        den[c] = d;
        obj[c] = d != 0.0 ? make_double2(num.x / d, -num.y / d) : make_double2(0, 0);
    }
    if (threadIdx.x == 0) {
        double nv = 0;
        for (int j = 0; j < cnt; ++j) nv += kp.statNoise[g0 + j] * kp.statNoise[g0 + j];
        noiseVar = cnt ? nv / cnt : 0.0;
    }
    __syncthreads();
    if (!ra.noFilter && cnt) {
        const double noiseFactor = noiseVar * N * N;
        for (int c = threadIdx.x; c < N2; c += THREADS)
            tmp[c] = (obj[c].x * obj[c].x + obj[c].y * obj[c].y) * den[c];
        __syncthreads();
        restore_smooth<N, THREADS>(tmp, pt, 1, 1);
        for (int c = threadIdx.x; c < N2; c += THREADS) pt[c] = noiseFactor / pt[c];
        __syncthreads();
        // rr(y, x) = max(1 - (pt(-y, -x) + pt(y, x)) / 2, 0), clipped to {0} u [0.2, 1]
        for (int c = threadIdx.x; c < N2; c += THREADS) {
            const int y = c / N, x = c % N;
            double v = 1.0 - 0.5 * (pt[((N - y) % N) * N + (N - x) % N] + pt[c]);
            v = v > 0.0 ? v : 0.0;
            if (v < 0.2) v = 0.0;
            if (v > 1.0) v = 1.0;
            if (c == (N / 2) * N + N / 2) v = 1.0;     // DC gain = 1
            rr[c] = v;
            mask[c] = (c == (N / 2) * N + N / 2) ? 1 : 0;
        }
        __syncthreads();
        // connectedRegion: the 4-connected region of rr > 0 around the centre, grown until it
        // stops changing (at most N * N sweeps)
        for (int it = 0; it < N2; ++it) {
            if (threadIdx.x == 0) changed = 0;
            __syncthreads();
            int any = 0;
            for (int c = threadIdx.x; c < N2; c += THREADS) {
                if (mask[c] || !(rr[c] > 0.0)) continue;
                const int y = c / N, x = c % N;
                if ((y > 0 && mask[c - N]) || (y < N - 1 && mask[c + N]) || (x > 0 && mask[c - 1]) ||
                    (x < N - 1 && mask[c + 1])) {
                    mask[c] = 1;
                    any = 1;
                }
            }
            if (any) changed = 1;
            __syncthreads();
            if (!changed) break;
        }
        for (int c = threadIdx.x; c < N2; c += THREADS) rr[c] = mask[c] ? rr[c] : 0.0;
        __syncthreads();
        restore_smooth<N, THREADS>(rr, tmp, 4, 4);
        const double fc = 0.9 * ra.fc[o];
        const double fc2 = fc * fc;
        for (int c = threadIdx.x; c < N2; c += THREADS) {
            const int y = c / N, x = c % N;
            const double r2 = (double)(y - N / 2) * (y - N / 2) + (double)(x - N / 2) * (x - N / 2);
            obj[c] = r2 > fc2 ? make_double2(0, 0) : make_double2(obj[c].x * tmp[c], obj[c].y * tmp[c]);
        }
        __syncthreads();
    }
    // ift: un-centre, backward transform, real part / N^2.  The rows and then the columns
    // are transformed in bands of Band<N> lines through shared memory (an N x N FP64
    // tile does not fit for N = 128); the row results go to W (the den and pt arrays).
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int B = Band<N>::value;
    static_assert(N % B == 0, "bands tile the array");
    cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);     // [B][LDS]
    cx<double>* tw = s + B * LDS;
    cx<double>* W = reinterpret_cast<cx<double>*>(den);
    for (int k = threadIdx.x; k < N; k += THREADS) {
        double sn, cs;
        sincospi(2.0 * k / N, &sn, &cs);
        tw[k] = mkc<double>(cs, -sn);
    }
    for (int r0 = 0; r0 < N; r0 += B) {
        __syncthreads();
        for (int i = threadIdx.x; i < B * N; i += THREADS) {
            const int y = r0 + i / N, x = i % N;
            const double2 v = obj[((y + N / 2) % N) * N + (x + N / 2) % N];
            s[(i / N) * LDS + x] = mkc<double>(v.x, v.y);
        }
        __syncthreads();
        fft_lines<double, N, +1, B, true, THREADS>(s, 0, tw, threadIdx.x);
        for (int i = threadIdx.x; i < B * N; i += THREADS) W[(r0 + i / N) * N + i % N] = s[(i / N) * LDS + i % N];
    }
    const int ps = kp.ps, off = (N - ps) / 2;
    float* out = ra.out + ((size_t)p * kp.nObj + o) * ps * ps;
    for (int c0 = 0; c0 < N; c0 += B) {
        __syncthreads();
        for (int i = threadIdx.x; i < B * N; i += THREADS) {
            const int col = c0 + i % B, y = i / B;
            s[(i % B) * LDS + y] = W[y * N + col];
        }
        __syncthreads();
        fft_lines<double, N, +1, B, true, THREADS>(s, 0, tw, threadIdx.x);
        for (int i = threadIdx.x; i < B * N; i += THREADS) {
            const int x = c0 + i / N, y = i % N;
            const float v = (float)(s[(i / N) * LDS + y].x / (double)N2);
            if (x >= off && x < off + ps && y >= off && y < off + ps) out[(y - off) * ps + (x - off)] = v;
            if (ra.objFull) ra.objFull[(size_t)b * N2 + y * N + x] = v;
        }
    }
}

// Per (patch, object): the unnormalised transform of the float object (the convolution of
// SubImage::convolveImage transforms ObjectData::img, fouriertransform.hpp:310-324) and, for
// kRestorePsfAvg, the mean PSF of the object's images (SubImage::addPSF summed in image order
// in FP64, stored as float and scaled by 1/count, object.cpp:345-350).
template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_restore_objft(KParams<T> kp, RestoreOutArgs oa) {
    constexpr int N2 = N * N, LDS = Tile<N>::LDS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);
    cx<double>* tw = s + kRestoreBand * LDS;
    restore_twiddles<N, THREADS>(tw);
    cx<double>* W = reinterpret_cast<cx<double>*>(oa.pool + (size_t)blockIdx.x * 3 * N2);
    double* acc = oa.pool + (size_t)blockIdx.x * 3 * N2 + 2 * N2;
    const int ps = kp.ps, off = (N - ps) / 2;
    for (int b = blockIdx.x; b < kp.P * kp.nObj; b += gridDim.x) {
        const float* img = oa.objFull + (size_t)b * N2;
        cx<double>* F = oa.Fo + (size_t)b * N2;
        fft2_banded<N, -1, THREADS>([&](int y, int x) { return mkc<double>((double)img[y * N + x], 0.0); },
                                    [&](int y, int x, cx<double> v) { F[y * N + x] = v; }, W, s, tw);
        if (!(oa.flags & kRestorePsfAvg)) continue;
        const int p = b / kp.nObj, o = b % kp.nObj;
        const int first = kp.pObjFirst[b], cnt = kp.pObjCount[b];
        for (int c = threadIdx.x; c < N2; c += THREADS) acc[c] = 0.0;
        for (int j = 0; j < cnt; ++j) {
            const cx<T>* S = kp.S + ((size_t)p * kp.I + first + j) * N2;
            // PSF = reorder(real(ift(reorder(OTF))) / N^2) (OTF flags REORDER_IMG|REORDER_FT|
            // NORMALIZE_FT, subimage.cpp:89-90, 615-626)
            fft2_banded<N, +1, THREADS>(
                [&](int y, int x) {
                    const cx<T> v = S[((y + N / 2) % N) * N + (x + N / 2) % N];
                    return mkc<double>((double)v.x, (double)v.y);
                },
                [&](int y, int x, cx<double> v) {
                    acc[((y + N / 2) % N) * N + (x + N / 2) % N] += v.x / (double)N2;
                },
                W, s, tw);
        }
        float* out = oa.psf + (size_t)b * ps * ps;
        const double inv = 1.0 / cnt;
        for (int c = threadIdx.x; c < ps * ps; c += THREADS) {
            const int y = c / ps + off, x = c % ps + off;
            out[c] = (float)((double)(float)acc[y * N + x] * inv);
        }
        __syncthreads();
    }
}

// Per image: the PSF (SubImage::getPSF), the convolved object (SubImage::convolveImage of the
// float object: real(ift(ft(img) / N^2 * OTF)) with the OTF un-centred) and the residual
// (convolved object as float minus the image, SubImage::convolvedResidual / residual,
// subimage.hpp:110-129, the image being real(ift(D)) / N^2, the windowed and padded cutout).
template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_restore_images(KParams<T> kp, RestoreOutArgs oa) {
    constexpr int N2 = N * N, LDS = Tile<N>::LDS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);
    cx<double>* tw = s + kRestoreBand * LDS;
    restore_twiddles<N, THREADS>(tw);
    cx<double>* W = reinterpret_cast<cx<double>*>(oa.pool + (size_t)blockIdx.x * 3 * N2);
    double* img = oa.pool + (size_t)blockIdx.x * 3 * N2 + 2 * N2;
    const int ps = kp.ps, off = (N - ps) / 2;
    auto trimmed = [&](int y, int x) { return y >= off && y < off + ps && x >= off && x < off + ps; };
    for (int g = blockIdx.x; g < kp.P * kp.I; g += gridDim.x) {
        const int p = g / kp.I, j = g % kp.I, o = kp.pImgObj[g];
        if (j >= kp.pgeo[p].nImg) continue;   // an image slot the patch does not use
        const cx<T>* S = kp.S + (size_t)g * N2;
        auto otfU = [&](int y, int x) {   // the OTF with the zero frequency at (0, 0)
            const cx<T> v = S[((y + N / 2) % N) * N + (x + N / 2) % N];
            return mkc<double>((double)v.x, (double)v.y);
        };
        if (oa.flags & kRestorePsf) {
            float* out = oa.psf + (size_t)g * ps * ps;
            fft2_banded<N, +1, THREADS>(otfU,
                                        [&](int y, int x, cx<double> v) {
                                            const int yy = (y + N / 2) % N, xx = (x + N / 2) % N;
                                            if (trimmed(yy, xx))
                                                out[(yy - off) * ps + (xx - off)] = (float)(v.x / (double)N2);
                                        },
                                        W, s, tw);
        }
        if (!(oa.flags & (kRestoreCobj | kRestoreResidual))) continue;
        if (oa.flags & kRestoreResidual) {
            const cx<T>* D = kp.D + (size_t)g * N2;
            fft2_banded<N, +1, THREADS>(
                [&](int y, int x) {
                    const cx<T> v = D[((y + N / 2) % N) * N + (x + N / 2) % N];
                    return mkc<double>((double)v.x, (double)v.y);
                },
                [&](int y, int x, cx<double> v) { img[y * N + x] = v.x / (double)N2; }, W, s, tw);
        }
        const cx<double>* F = oa.Fo + ((size_t)p * kp.nObj + o) * N2;
        float* co = oa.cobj ? oa.cobj + (size_t)g * ps * ps : nullptr;
        float* re = oa.res ? oa.res + (size_t)g * ps * ps : nullptr;
        fft2_banded<N, +1, THREADS>(
            [&](int y, int x) {
                const cx<double> f = F[y * N + x], t = otfU(y, x);
                return mkc<double>(f.x * t.x - f.y * t.y, f.x * t.y + f.y * t.x);
            },
            [&](int y, int x, cx<double> v) {
                if (!trimmed(y, x)) return;
                const float c = (float)(v.x / (double)N2);
                const int q = (y - off) * ps + (x - off);
                if ((oa.flags & kRestoreCobj) && co) co[q] = c;
                if ((oa.flags & kRestoreResidual) && re) re[q] = (float)((double)c - img[y * N + x]);
            },
            W, s, tw);
    }
}

}  // namespace rdxg
