// Per-image and per-object kernels of the batched MOMFBD solver.
//
// Data layout in device memory (g = patch * I + image, po = patch * nObj + object):
//   D  [g][N*N]  complex  centred transform of the windowed image (SubImage::imgFT)
//   S  [g][N*N]  complex  centred OTF (SubImage::OTF)
//   X  [g][N*N]  complex  un-centred transform of c * pupil function (kept for gradients)
//   PF [g][n*n]  complex  pupil function A exp(i phi) (SubImage::PF)
//   O  [po][N*N] complex  object estimate conj(P)/Q (centred)
//   Qt [po][N*N] real     Q = gamma + sum |S|^2
// Every per-image kernel runs one thread block per image over an N x N shared-memory
// tile; patches whose request does not need the kernel return at once.
#pragma once

#include "cg_machine.h"
#include "rdxg_fft.cuh"

namespace rdxg {

// Geometry of one patch of the batch.  A uniform batch gives every patch the handle's own;
// a ragged batch (rdxg_set_patch_shapes) gives each patch its frames per channel and its
// modes: its images fill the first nImg image slots (each channel's first frames, in the
// handle's image order) and its modes are the first nMode of the handle's.
struct PatchGeo {
    int32_t nImg;       // image slots in use, [0, nImg)
    int32_t nMode;      // modes in use, [0, nMode)
    int32_t nFree;      // columns of its null-space map
    int32_t chunks;     // chunks of its images in the fused evaluation
    int32_t rowBase;    // its null-space map by row: rowPtr[rowBase + r], r < I*M (handle rows)
    int32_t colBase;    // by column: colPtr[colBase + c], c <= nFree
};

template <typename T>
struct KParams {
    int32_t P, I, M, nObj, N, n, ps, cs, margin, nTiles;
    // static
    const T* Z;          // [M][n*n]
    const T* A;          // [n*n] amplitude, zero outside the pupil support
    const T* phiFixed;   // [C][n*n]
    const T* otfNorm;    // [C]
    const uint8_t* otfMask;   // [N*N] centred OTF support
    const PatchGeo* pgeo;     // [P]
    const int32_t* pImgObj;   // [P][I] object of each image slot of each patch
    const int32_t* pImgCh;    // [P][I] channel of each image slot
    const int32_t* pObjFirst; // [P][nObj] first image slot of each object
    const int32_t* pObjCount; // [P][nObj]
    const double* objWeight;  // [nObj]
    const double* objGradStep;// [nObj]
    const double* window;     // [ps*ps]
    const double* noiseWindow;// [ps*ps]
    const cx<T>* tw;          // [N] exp(-2 pi i k/N)
    double area;
    // the adjoint's factor per object and channel, [2][nObj][nCh]: Vogel, exact gradient
    // (formed on the host, so that no block spends GB300's narrow FP64 pipe on it)
    const double* gradScale;
    int32_t nCh;
    int32_t tiltX, tiltY;
    // per patch
    const float* cutouts;     // [g][cs*cs]
    int32_t* shift;           // [g][2] (y, x)
    double* statMean;         // [g]
    double* statStd;          // [g]
    double* statNoise;        // [g]
    double* rg;               // [g] noise / stddev
    const T* alphaEff;        // [g][M]
    cx<T>* D;
    cx<T>* S;
    cx<T>* X;
    cx<T>* PF;
    cx<T>* O;
    T* Qt;
    const double* gamma;      // [po]
    double* partial;          // [po][nTiles]
    double* galpha;           // [g][M]
    const int32_t* req;       // [P]
    const int32_t* gmethod;   // [P]
    const int32_t* modeCount; // [P]
    const uint8_t* reinit;    // [g] image must be re-initialised (re-shift)
    // patches whose gradient is requested this round (built by the solver kernel)
    const int32_t* gradP;     // [P] analytic gradient
    const int32_t* nGradP;
    const int32_t* fdP;       // [P] finite-difference gradient
    const int32_t* nFdP;
    // half-plane copy of D for the fused evaluation (null when unused)
    cx<T>* Dh;                // [g][nH]
    const int32_t* hIdx;      // [nH] centred indices
    int32_t nH;
    // fitted planes (FIT_PLANE): [po][2] slopes (a along y, b along x) of the plane fitted to
    // the object's mean image, or null
    double* plane;
    // launch-shape variants picked by the planner (read by the host-side launchers only):
    // 0 the default block size, 1 the alternative (see rdxg_launch.h)
    int32_t shapeEval, shapeFwd, shapeAdj;
    // Recomputed transforms: X and PF (and on the fused path S) are not kept between the
    // evaluation and the gradient kernels, which form them again from the phases.
    int32_t recompute;
    // [g][n*n] phases of this evaluation when the mode expansion ran before the transforms
    // (the fused path, and the tensor-core expansion on the general path); null: the
    // transform kernels form phi_fixed + sum alpha Z themselves
    const T* phiImg;
    cx<T>* Xscr;              // [slot][N*N] scratch of the recomputing kernels
    int32_t scrBlocks;        // blocks of the persistent ones (slot = block)
    unsigned* slotMask;       // [SM] slots in use, for the kernels with one item per block
    int32_t slotsPerSM;
    int32_t* rcStatus;        // non-zero: a block found no free slot
    // per-block N x N work tiles in global memory, for the sizes whose tile does not fit a
    // block's shared memory (GlobalTile: FP64 at N = 128); blocks of the tile kernels
    cx<T>* gtile;
    int32_t gtileBlocks;
};

// FP64 at N = 128: a double tile of 128 x 129 (264 KB) exceeds the 227 KB of shared memory
// of a block, so the general path's transform kernels keep their tile in global memory (one
// per block, L2-resident) and only the twiddles and small arrays in shared memory.  The
// transforms are the same code (generic pointers, block barriers order global memory too).
template <typename T, int N> struct GlobalTile {
    static constexpr bool value = (size_t)(Tile<N>::ELEMS + N) * sizeof(cx<T>) > 227 * 1024;
};
// the block's work tile and the start of its shared-memory arrays (twiddles first)
template <typename T, int N>
__device__ __forceinline__ cx<T>* work_tile(const KParams<T>& kp, unsigned char* smem) {
    if constexpr (GlobalTile<T, N>::value) return kp.gtile + (size_t)blockIdx.x * Tile<N>::ELEMS;
    else return reinterpret_cast<cx<T>*>(smem);
}
template <typename T, int N>
__device__ __forceinline__ cx<T>* after_tile(unsigned char* smem) {
    if constexpr (GlobalTile<T, N>::value) return reinterpret_cast<cx<T>*>(smem);
    else return reinterpret_cast<cx<T>*>(smem) + Tile<N>::ELEMS;
}

enum GradKind : int32_t { GK_VOGEL = 0, GK_EXACT = 1 };

template <typename T> __device__ __forceinline__ void sincos_t(T x, T* s, T* c);
template <> __device__ __forceinline__ void sincos_t<float>(float x, float* s, float* c) { sincosf(x, s, c); }
template <> __device__ __forceinline__ void sincos_t<double>(double x, double* s, double* c) { sincos(x, s, c); }

// deterministic block reduction of a double (fixed tree); result valid in all threads
template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        double t = (lane < THREADS / 32) ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    double r = red[32];
    __syncthreads();
    return r;
}

template <typename T, int N>
__device__ __forceinline__ void load_twiddles(cx<T>* tw, const cx<T>* src) {
    for (int k = threadIdx.x; k < N; k += blockDim.x) tw[k] = src[k];
}

template <typename T, int N>
__device__ __forceinline__ void zero_tile(cx<T>* s) {
    for (int i = threadIdx.x; i < Tile<N>::ELEMS; i += blockDim.x) s[i] = mkc<T>(0, 0);
}

// The fitted plane at pixel (y, x) of the patch, as redux stores it: makePlane
// (image/utils.cpp:128-147) with the constant dropped (fitPlane(..., subtract_mean = true),
// object.cpp:588), centred at (ps/2, ps/2), rounded to float (Object::fittedPlane is float).
__device__ __forceinline__ double plane_value(const double* pl, int ps, int y, int x) {
    return (double)(float)(pl[0] * (double)(y - ps / 2) + pl[1] * (double)(x - ps / 2));
}

// ----------------------------------------------------------------------------------
// FIT_PLANE: Object::fitAvgPlane (object.cpp:553-594).  The object's images (the patch
// views of the cutouts at their current shifts) are averaged in float, in image order, and
// divided by their count in float; a plane z = a dy + b dx + c (dy = y - ps/2, dx = x - ps/2)
// is fitted to the mean image by least squares over every pixel (fitPlane, image/utils.cpp:
// 169-233, there by GSL's multifit; here by the 3x3 normal equations in double) and a, b
// kept.  One block per (patch, object); with full = 0 only objects with a re-initialised
// image are refitted (Object::reInitialize, object.cpp:885-904).
// ----------------------------------------------------------------------------------
template <typename T, int THREADS>
__global__ void __launch_bounds__(THREADS) k_fit_plane(KParams<T> kp, int full) {
    const int po = blockIdx.x;
    const int p = po / kp.nObj, o = po % kp.nObj;
    const int j0 = kp.pObjFirst[po], cnt = kp.pObjCount[po];
    __shared__ double red[33];
    __shared__ int any;
    if (!full) {
        if (threadIdx.x == 0) any = 0;
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += THREADS)
            if (kp.reinit[(size_t)p * kp.I + j0 + k]) any = 1;
        __syncthreads();
        if (!any) return;
    }
    const int ps = kp.ps, cs = kp.cs;
    double sz = 0, szy = 0, szx = 0;
    for (int i = threadIdx.x; i < ps * ps; i += THREADS) {
        const int y = i / ps, x = i % ps;
        float acc = 0.f;
        for (int k = 0; k < cnt; ++k) {
            const size_t g = (size_t)p * kp.I + j0 + k;
            const int oy = kp.margin + kp.shift[2 * g + 0], ox = kp.margin + kp.shift[2 * g + 1];
            acc = __fadd_rn(acc, kp.cutouts[g * cs * cs + (size_t)(oy + y) * cs + ox + x]);
        }
        const double z = (double)__fdiv_rn(acc, (float)cnt);
        sz += z;
        szy += z * (double)(y - ps / 2);
        szx += z * (double)(x - ps / 2);
    }
    const double tz = block_sum<THREADS>(sz, red);
    const double tzy = block_sum<THREADS>(szy, red);
    const double tzx = block_sum<THREADS>(szx, red);
    if (threadIdx.x == 0) {
        // normal equations over the full grid: dy and dx run over [-ps/2, ps - 1 - ps/2]
        double s1 = 0, s2 = 0;
        for (int v = 0; v < ps; ++v) {
            const double d = (double)(v - ps / 2);
            s1 += d;
            s2 += d * d;
        }
        const double n = (double)ps;
        // [ n s2  s1^2  n s1 ] [a]   [ tzy ]
        // [ s1^2  n s2  n s1 ] [b] = [ tzx ]
        // [ n s1  n s1  n^2  ] [c]   [ tz  ]
        const double A[3][3] = {{n * s2, s1 * s1, n * s1}, {s1 * s1, n * s2, n * s1}, {n * s1, n * s1, n * n}};
        const double rhs[3] = {tzy, tzx, tz};
        auto det3 = [](const double m[3][3]) {
            return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                   m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
        };
        const double d0 = det3(A);
        double sol[2];
        for (int c = 0; c < 2; ++c) {
            double B[3][3];
            for (int r = 0; r < 3; ++r)
                for (int q = 0; q < 3; ++q) B[r][q] = (q == c) ? rhs[r] : A[r][q];
            sol[c] = det3(B) / d0;
        }
        kp.plane[2 * (size_t)po + 0] = sol[0];
        kp.plane[2 * (size_t)po + 1] = sol[1];
    }
}

// od.img += fittedPlane after the restoration (object.cpp:410-413): objects [po][ps][ps].
template <int UNUSED = 0>
__global__ void k_add_plane(const double* plane, float* objects, int ps) {
    const int po = blockIdx.x;
    const double* pl = plane + 2 * (size_t)po;
    float* ob = objects + (size_t)po * ps * ps;
    for (int i = threadIdx.x; i < ps * ps; i += blockDim.x)
        ob[i] = __fadd_rn(ob[i], (float)plane_value(pl, ps, i / ps, i % ps));
}

// ----------------------------------------------------------------------------------
// Image preparation: SubImage::initialize (subimage.cpp:155-209) with getWindowedImg
// (106-150) and the noise estimate FourierTransform::noise(-1,-1) (fouriertransform.cpp:
// 448-495).  mode 1: full initialisation (noise and rg); mode 0: re-initialise only the
// images flagged in reinit (after a re-shift).
// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_prep(KParams<T> kp, int full) {
    const int g = blockIdx.x;
    if (g % kp.I >= kp.pgeo[g / kp.I].nImg) return;   // an image slot the patch does not use
    if (!full && !kp.reinit[g]) return;
    constexpr int LDS = Tile<N>::LDS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* s = work_tile<T, N>(kp, smem_raw);
    cx<T>* tw = after_tile<T, N>(smem_raw);
    double* red = reinterpret_cast<double*>(tw + N);
    load_twiddles<T, N>(tw, kp.tw);
    const int ps = kp.ps, cs = kp.cs;
    const int oy = kp.margin + kp.shift[2 * g + 0];
    const int ox = kp.margin + kp.shift[2 * g + 1];
    const float* cut = kp.cutouts + (size_t)g * cs * cs;
    // FIT_PLANE: getWindowedImg subtracts the object's fitted plane inside the window,
    // (img - avg - plane) * window + avg (subimage.cpp:117-123)
    const double* pl = kp.plane ? kp.plane + 2 * ((size_t)(g / kp.I) * kp.nObj + kp.pImgObj[g]) : nullptr;
    auto windowed = [&](int y, int x, int i, double avg) {
        const double v = (double)cut[(oy + y) * cs + ox + x] - avg;
        return (pl ? v - plane_value(pl, ps, y, x) : v) * kp.window[i] + avg;
    };
    // raw mean
    double sum = 0;
    for (int i = threadIdx.x; i < ps * ps; i += THREADS) {
        const int y = i / ps, x = i % ps;
        sum += (double)cut[(oy + y) * cs + ox + x];
    }
    const double avg = block_sum<THREADS>(sum, red) / (double)(ps * ps);
    // windowed image statistics
    double s1 = 0, s2 = 0;
    for (int i = threadIdx.x; i < ps * ps; i += THREADS) {
        const int y = i / ps, x = i % ps;
        const double w = windowed(y, x, i, avg);
        s1 += w;
        s2 += w * w;
    }
    const double t1 = block_sum<THREADS>(s1, red);
    const double t2 = block_sum<THREADS>(s2, red);
    const double mean = t1 / (double)(ps * ps);
    const double stddev = sqrt(t2 / (double)(ps * ps) - mean * mean);
    if (full) {
        // noise estimate from (windowed - mean) * noiseWindow, un-centred transform
        for (int i = threadIdx.x; i < N * N; i += THREADS) {
            const int y = i / N, x = i % N;
            const double w = windowed(y, x, i, avg);
            s[y * LDS + x] = mkc<T>((T)((w - mean) * kp.noiseWindow[i]), 0);
        }
        __syncthreads();
        fft2d<T, N, -1, THREADS, false>(s, tw);
        const int mask = N / 6 + 1;
        const double limits = (double)N * N / 4.0;
        double np = 0, cnt = 0;
        for (int i = threadIdx.x; i < N * N; i += THREADS) {
            const int y = i / N, x = i % N;
            if (x < mask || x >= N - mask + 1 || y < mask || y >= N - mask + 1) continue;
            const double xx = (double)(x < N - x ? x : N - x);
            const double yy = (double)(y < N - y ? y : N - y);
            if (xx * xx + yy * yy < limits) continue;
            const cx<T> v = s[y * LDS + x];
            np += (double)v.x * v.x + (double)v.y * v.y;
            cnt += 1.0;
        }
        const double tp = block_sum<THREADS>(np, red);
        const double tc = block_sum<THREADS>(cnt, red);
        const double noise = tc > 0 ? sqrt(tp / (tc * N * N)) : 0.0;
        if (threadIdx.x == 0) {
            kp.statNoise[g] = noise;
            kp.rg[g] = noise / stddev;
        }
    }
    if (threadIdx.x == 0) {
        kp.statMean[g] = mean;
        kp.statStd[g] = stddev;
    }
    // D = FT(windowed) = FT(windowed - mean) + N^2 mean delta: the mean is taken out before
    // the transform so that the large DC term does not swamp the other frequencies.
    for (int i = threadIdx.x; i < N * N; i += THREADS) {
        const int y = i / N, x = i % N;
        const double w = windowed(y, x, i, avg);
        s[y * LDS + x] = mkc<T>((T)(w - mean), 0);
    }
    __syncthreads();
    fft2d<T, N, -1, THREADS, false>(s, tw);
    cx<T>* D = kp.D + (size_t)g * N * N;
    const cx<T> dc = mkc<T>((T)(mean * (double)N * (double)N), 0);
    for (int i = threadIdx.x; i < N * N; i += THREADS) {
        const int cy = i / N, cxx = i % N;          // centred index (REORDER_FT)
        const int y = (cy + N / 2) % N, x = (cxx + N / 2) % N;
        D[i] = (y == 0 && x == 0) ? dc : s[y * LDS + x];
    }
    if (kp.Dh) {
        for (int h = threadIdx.x; h < kp.nH; h += THREADS) {
            const int c = kp.hIdx[h];
            const int y = (c / N + N / 2) % N, x = (c % N + N / 2) % N;
            kp.Dh[(size_t)g * kp.nH + h] = (y == 0 && x == 0) ? dc : s[y * LDS + x];
        }
    }
}

// ----------------------------------------------------------------------------------
// Forward model: SubImage::calcPhi + calcPFOTF (subimage.cpp:509-544, 586-612).
// phi = phi_fixed + sum_m alpha_eff[m] Z_m; PF = A exp(i phi);
// OTF = fftshift(ifft(|fft(c PF embedded at n/2)|^2) / N^2).
// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS, typename PL = Plan<N>>
__global__ void __launch_bounds__(THREADS) k_forward(KParams<T> kp) {
    const int g = blockIdx.x;
    const int p = g / kp.I, j = g % kp.I;
    const int rq = kp.req[p];
    if (rq != REQ_F && rq != REQ_DF) return;
    if (j >= kp.pgeo[p].nImg) return;
    // X and PF are kept for the gradient kernels unless they recompute them
    const bool df = (rq == REQ_DF) && !kp.recompute;
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* s = work_tile<T, N>(kp, smem_raw);
    cx<T>* tw = after_tile<T, N>(smem_raw);
    T* al = reinterpret_cast<T*>(tw + N);
    load_twiddles<T, N>(tw, kp.tw);
    const int M = kp.M;
    for (int m = threadIdx.x; m < M; m += THREADS) al[m] = kp.alphaEff[(size_t)g * M + m];
    zero_tile<T, N>(s);
    __syncthreads();
    const int ch = kp.pImgCh[g];
    const T c = kp.otfNorm[ch];
    const T* phf = kp.phiFixed + (size_t)ch * n2;
    for (int q = threadIdx.x; q < n2; q += THREADS) {
        const T a = kp.A[q];
        cx<T> pf = mkc<T>(0, 0);
        if (a > (T)0) {
            T phi;
            if (kp.phiImg) {
                phi = kp.phiImg[(size_t)g * n2 + q];     // expanded on the tensor cores (k_phase_tc)
            } else {
                phi = phf[q];
                for (int m = 0; m < M; ++m) phi += al[m] * kp.Z[(size_t)m * n2 + q];
            }
            T sn, cs;
            sincos_t<T>(phi, &sn, &cs);
            pf = mkc<T>(a * cs, a * sn);
        }
        if (df) kp.PF[(size_t)g * n2 + q] = pf;
        const int y = q / n, x = q % n;
        s[(y + n / 2) * LDS + x + n / 2] = cscale<T>(pf, c);
    }
    __syncthreads();
    fft2d<T, N, -1, THREADS, true, PL>(s, tw);
    cx<T>* X = kp.X + (size_t)g * N * N;
    for (int i = threadIdx.x; i < N * N; i += THREADS) {
        const int y = i / N, x = i % N;
        const cx<T> v = s[y * LDS + x];
        if (df) X[i] = v;
        s[y * LDS + x] = mkc<T>(cnorm<T>(v), 0);
    }
    __syncthreads();
    fft2d<T, N, +1, THREADS, false, PL>(s, tw);
    const T inv = (T)1 / (T)(N * N);
    cx<T>* S = kp.S + (size_t)g * N * N;
    for (int i = threadIdx.x; i < N * N; i += THREADS) {
        const int cy = i / N, cxx = i % N;
        const int y = (cy + N / 2) % N, x = (cxx + N / 2) % N;
        S[i] = cscale<T>(s[y * LDS + x], inv);
    }
}

// ----------------------------------------------------------------------------------
// Per-object accumulation and metric: Object::initPQ/addToPQ/calcMetric
// (object.cpp:459-518, 597-615).  The reference's per-frequency term
//     sum_j |D_j|^2 - |P|^2 / Q,   P = sum_j conj(D_j) S_j,  Q = gamma + sum_j |S_j|^2
// is a small difference of large numbers.  With O = conj(P) / Q it equals exactly
//     sum_j |D_j - O S_j|^2 + gamma |O|^2,
// a sum of non-negative terms, which is what is evaluated here (two passes over the
// object's images per frequency; the second pass hits L2).  Per-block partial sums are in
// double and are added in a fixed order by the solver kernel.
// ----------------------------------------------------------------------------------
template <typename T, int THREADS>
__global__ void __launch_bounds__(THREADS) k_accum(KParams<T> kp) {
    const int po = blockIdx.y;
    const int p = po / kp.nObj, o = po % kp.nObj;
    const int rq = kp.req[p];
    if (rq != REQ_F && rq != REQ_DF) return;
    __shared__ double red[33];
    const int N2 = kp.N * kp.N;
    const int u = blockIdx.x * THREADS + threadIdx.x;
    double term = 0;
    const bool df = (rq == REQ_DF);
    if (u < N2) {
        const size_t fbase = (size_t)p * kp.I + kp.pObjFirst[po];
        const int cnt = kp.pObjCount[po];
        const T gam = (T)kp.gamma[po];
        cx<T> O = mkc<T>(0, 0);
        T Qt = (T)1;
        if (kp.otfMask[u]) {
            cx<T> Pa = mkc<T>(0, 0);
            T Qa = (T)0;
            for (int k = 0; k < cnt; ++k) {
                const cx<T> d = kp.D[(fbase + k) * N2 + u];
                const cx<T> sv = kp.S[(fbase + k) * N2 + u];
                Pa = cadd<T>(Pa, cmulc<T>(sv, d));          // conj(D) S
                Qa += cnorm<T>(sv);
            }
            Qt = gam + Qa;
            O = mkc<T>(Pa.x / Qt, -Pa.y / Qt);             // conj(P) / Q
            T R = (T)0;
            for (int k = 0; k < cnt; ++k) {
                const cx<T> d = kp.D[(fbase + k) * N2 + u];
                const cx<T> sv = kp.S[(fbase + k) * N2 + u];
                const cx<T> r = csub<T>(d, cmul<T>(O, sv));
                R += cnorm<T>(r);
            }
            term = (double)R + (double)gam * (double)cnorm<T>(O);
        }
        if (df) {
            kp.O[(size_t)po * N2 + u] = O;
            kp.Qt[(size_t)po * N2 + u] = Qt;
        }
    }
    const double tot = block_sum<THREADS>(term, red);
    if (threadIdx.x == 0) kp.partial[(size_t)po * kp.nTiles + blockIdx.x] = tot;
}

// a + b = s + e exactly (Knuth's TwoSum), in FP32 with explicit roundings
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (hi, lo) += (h2, l2) as float-float numbers (about 48 significant bits)
__device__ __forceinline__ void ff_add(float& hi, float& lo, float h2, float l2) {
    float s, e;
    two_sum(hi, h2, s, e);
    e = __fadd_rn(e, __fadd_rn(lo, l2));
    two_sum(s, e, hi, lo);
}
// Float-float sum over the warp by a fixed shuffle tree; lane 0 holds the total.  Sums that the
// path used to form in FP64 are formed this way on the FP32 pipe (GB300 issues an FP64
// instruction, conversions included, at a small fraction of the FP32 rate).
__device__ __forceinline__ void warp_sum_ff(float& hi, float& lo) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, hi, off);
        const float ol = __shfl_down_sync(0xffffffffu, lo, off);
        ff_add(hi, lo, oh, ol);
    }
}


// ----------------------------------------------------------------------------------
// Adjoint gradient: SubImage::calcVogelWeight + gradientVogel (subimage.cpp:312-390).
// With G = conj(O) (D - O S) = (PQ D - PS S) / QS on the OTF support, the reference forms
// U = fftshift(fft(ifft(corner-embedded PF)/N^2 * Re(ifft(ifftshift G)/N^2))) which is the
// convolution (G * PF)/N^2 on the pupil; here it is evaluated as
//     ifft( fft(ifftshift G) * fft(PF embedded at n/2) )
// where the second factor is the forward transform X kept from the forward pass (two
// transforms instead of three).  The DC term of G is left out: G(0) is real and its exact
// contribution Im(conj(PF) G(0) PF) is zero, while its size would swamp the FP32 result.
// kind GK_VOGEL: the reference's weights (pupil amplitude per pixel, -2 area/N^2, object
// weight twice); GK_EXACT: dL/dalpha of the metric.
// ----------------------------------------------------------------------------------
// The last step of the adjoint for image j of patch p: U = tile rows and columns [N/4, 3N/4)
// (the pupil), v = Im(conj(PF) U) times the pupil weight, and its projection on the enabled
// modes, one warp per mode (calcVogelWeight's last lines and gradientVogel,
// subimage.cpp:312-326, 376-389).  v: n^2 values of shared memory on a 16-byte boundary.
template <typename T, int N, int THREADS>
__device__ __forceinline__ void project_modes(const KParams<T>& kp, int kind, int p, int j, const cx<T>* s,
                                              const cx<T>* PF, T* v, int tid) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    const size_t g = (size_t)p * kp.I + j;
    const int o = kp.pImgObj[g];
#pragma unroll 4
    for (int q = tid; q < n2; q += THREADS) {
        const int y = q / n, x = q % n;
        const cx<T> U = s[(y + n / 2) * LDS + x + n / 2];
        const cx<T> pf = PF[q];
        // Im(conj(pf) U)
        const T a = kp.A[q];
        const T wq = (kind == GK_VOGEL) ? a : (a > (T)0 ? (T)1 : (T)0);
        v[q] = (pf.x * U.y - pf.y * U.x) * wq;
    }
    __syncthreads();
    // projection on the modes: one warp per mode, the lanes' partial sums added as float-float
    // numbers; then one thread per mode scales the total by the factor of the image's object
    // and channel
    const int lane = tid & 31, wid = tid >> 5;
    const int mc = kp.modeCount[p];
    const int ch = kp.pImgCh[g];
    float2* hl = reinterpret_cast<float2*>(v + n2);     // [M] the modes' sums (hi, lo)
    for (int m = wid; m < kp.M; m += THREADS / 32) {
        float hi = 0.f, lo = 0.f;
        if (m < mc) {
            const T* Zm = kp.Z + (size_t)m * n2;
            T part = 0;
            if constexpr (sizeof(T) == 4 && n2 % 4 == 0) {
                // four pixels per load (v and every mode row start on 16-byte boundaries: the
                // callers place v there and n2 * 4 bytes is a multiple of 16), so each lane has
                // a quarter of the loads of the scalar loop in flight at once
                const float4* Z4 = reinterpret_cast<const float4*>(Zm);
                const float4* v4 = reinterpret_cast<const float4*>(v);
#pragma unroll 4
                for (int q = lane; q < n2 / 4; q += 32) {
                    const float4 z = __ldg(Z4 + q), w = v4[q];
                    part += w.x * z.x + w.y * z.y + w.z * z.z + w.w * z.w;
                }
            } else {
#pragma unroll 8
                for (int q = lane; q < n2; q += 32) part += v[q] * Zm[q];
            }
            if constexpr (sizeof(T) == 4) {
                hi = (float)part;
                warp_sum_ff(hi, lo);
            } else {
                double acc = (double)part;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, off);
                if (lane == 0) reinterpret_cast<double*>(hl)[m] = acc;
            }
        }
        if (sizeof(T) == 4 && lane == 0) hl[m] = make_float2(hi, lo);
    }
    __syncthreads();
    const double scale = kp.gradScale[((size_t)(kind == GK_VOGEL ? 0 : 1) * kp.nObj + o) * kp.nCh + ch];
    for (int m = tid; m < kp.M; m += THREADS) {
        double acc;
        if constexpr (sizeof(T) == 4) acc = (double)hl[m].x + (double)hl[m].y;
        else acc = reinterpret_cast<const double*>(hl)[m];
        kp.galpha[g * kp.M + m] = (m < mc) ? acc * scale : 0.0;
    }
}

template <typename T, int N, int THREADS, typename PL = Plan<N>>
__device__ __forceinline__ void adjoint_image(const KParams<T>& kp, int kind, int p, int j) {
    const int g = p * kp.I + j;
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    constexpr bool PP = false;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* s = work_tile<T, N>(kp, smem_raw);
    cx<T>* s2 = s;
    cx<T>* tw = after_tile<T, N>(smem_raw);
    T* v = reinterpret_cast<T*>(tw + N);            // [n2]
    __syncthreads();    // previous image's shared memory consumed
    load_twiddles<T, N>(tw, kp.tw);
    const int o = kp.pImgObj[g];
    const size_t po = (size_t)p * kp.nObj + o;
    const cx<T>* Oo = kp.O + po * N2;
    const cx<T>* Dg = kp.D + (size_t)g * N2;
    const cx<T>* Sg = kp.S + (size_t)g * N2;
    bool halfG = false;
    if constexpr (sizeof(T) == 4 && N <= 88) halfG = kp.Dh != nullptr;
    if (halfG) {
        // fused path: G on the half plane, from the half-plane copy of D, and its mirror
        // G(-u) = conj G(u) (D, S, O are transforms of real images, so is G); half the loads
        for (int i = threadIdx.x; i < Tile<N>::ELEMS; i += THREADS) s[i] = mkc<T>(0, 0);
        __syncthreads();
        const cx<T>* Dh = kp.Dh + (size_t)g * kp.nH;
#pragma unroll 4
        for (int h = threadIdx.x; h < kp.nH; h += THREADS) {
            const int c = kp.hIdx[h];
            const int cy = c / N, cxx = c % N;
            const cx<T> O = Oo[c], D = Dh[h], S = Sg[c];
            const cx<T> G = cmulc<T>(csub<T>(D, cmul<T>(O, S)), O);   // conj(O) (D - O S)
            const int y = (cy + N / 2) % N, x = (cxx + N / 2) % N;      // un-centred (lag) position
            if (y == 0 && x == 0) continue;                                // the DC term is dropped
            s[y * LDS + x] = G;
            s[((N - y) % N) * LDS + (N - x) % N] = mkc<T>(G.x, -G.y);
        }
    } else {
        // unrolled, and the loads issued before the support test, so that each thread has
        // several iterations' global loads in flight in one round trip
#pragma unroll 8
        for (int i = threadIdx.x; i < N2; i += THREADS) {
            const int y = i / N, x = i % N;                 // un-centred (lag) position
            const int c = ((y + N / 2) % N) * N + (x + N / 2) % N;
            const uint8_t m = kp.otfMask[c];
            const cx<T> O = Oo[c], D = Dg[c], S = Sg[c];
            const cx<T> G = cmulc<T>(csub<T>(D, cmul<T>(O, S)), O);   // conj(O) (D - O S)
            s[y * LDS + x] = (m && !(y == 0 && x == 0)) ? G : mkc<T>(0, 0);
        }
    }
    __syncthreads();
    fft2d<T, N, -1, THREADS, false, PL>(s, tw);
    (void)s2;
    const cx<T>* X = kp.X + (size_t)g * N2;
#pragma unroll 8
    for (int i = threadIdx.x; i < N2; i += THREADS) {
        const int y = i / N, x = i % N;
        s[y * LDS + x] = cmul<T>(s[y * LDS + x], X[i]);
    }
    __syncthreads();
    if constexpr (PP) fft2d_pp_out_rows_pruned<T, N, +1, THREADS>(s, s2, tw);
    else fft2d_out_rows_pruned<T, N, +1, THREADS, PL>(s, tw);
    static_assert(((size_t)(Tile<N>::ELEMS + N) * sizeof(cx<T>)) % 16 == 0, "v is 16-byte aligned");
    const cx<T>* PF = kp.PF + (size_t)g * n2;
    project_modes<T, N, THREADS>(kp, kind, p, j, s, PF, v, (int)threadIdx.x);
}


template <typename T, int N, int THREADS, typename PL = Plan<N>>
__global__ void __launch_bounds__(THREADS) k_adjoint(KParams<T> kp, int kind) {
    // one work item per block (the grid covers every image of the batch): in a loop over
    // items the in-place transforms' index arithmetic is hoisted and spills
    const int nWork = *kp.nGradP * kp.I;
    const int w = blockIdx.x;
    if (w >= nWork) return;
    const int p = kp.gradP[w / kp.I], j = w % kp.I;
    if (j < kp.pgeo[p].nImg) adjoint_image<T, N, THREADS, PL>(kp, kind, p, j);
}

// The same kernel with registers for three 256-thread or two 512-thread blocks per SM, as many
// as their shared memory allows (FP32 up to N = 88): a round's ~700 gradient images take fewer
// waves.  (Where the bound would spill, at N = 128 and in FP64, k_adjoint is used.)
template <typename T, int N, int THREADS, typename PL = Plan<N>>
__global__ void __launch_bounds__(THREADS, THREADS == 256 ? 3 : 2) k_adjoint_mb(KParams<T> kp, int kind) {
    const int nWork = *kp.nGradP * kp.I;
    const int w = blockIdx.x;
    if (w >= nWork) return;
    const int p = kp.gradP[w / kp.I], j = w % kp.I;
    if (j < kp.pgeo[p].nImg) adjoint_image<T, N, THREADS, PL>(kp, kind, p, j);
}
template <typename T, int N, int THREADS, typename PL = Plan<N>>
constexpr auto adjoint_kernel() {
    if constexpr (sizeof(T) == 4 && N <= 88) return &k_adjoint_mb<T, N, THREADS, PL>;
    else return &k_adjoint<T, N, THREADS, PL>;
}

// ----------------------------------------------------------------------------------
// Recomputed transforms (KParams::recompute).  The reference keeps the pupil function and the
// OTF of every image (SubImage::PF, SubImage::OTF, subimage.hpp:156-158) from the metric
// evaluation to calcVogelWeight (subimage.cpp:348-371); here, when the per-image arrays of a
// batch would not fit the memory budget, the gradient kernels form them again from the
// phases: PF = A exp(i phi) and its transform X (and, on the fused path, which keeps no full
// OTF, S = ifft|X|^2 / N^2), so only the image transform D stays per image.  The phases are
// those of the evaluation (phiImg) or phi_fixed + sum alpha Z in the order of k_forward, so
// PF and X are the numbers the evaluation formed.  X lives in shared memory
// where two tiles fit (FP32 up to N = 88) and otherwise in a scratch slot of the SM the
// block runs on (acquire_slot).
// ----------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T image_phase(const KParams<T>& kp, const T* al, const T* phf, size_t g, int q, int n2) {
    if (kp.phiImg) return kp.phiImg[g * n2 + q];
    T phi = phf[q];
    for (int m = 0; m < kp.M; ++m) phi += al[m] * kp.Z[(size_t)m * n2 + q];
    return phi;
}

// PF of image g into pf (shared memory) and c PF embedded at n/2 in the zeroed tile s; al
// (shared memory) receives the image's coefficients first when the phases come from them.
template <typename T, int N, int THREADS>
__device__ __forceinline__ void recompute_pupil(const KParams<T>& kp, size_t g, int j, cx<T>* s, cx<T>* pf, T* al,
                                                int tid) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n;
    (void)j;
    const int ch = kp.pImgCh[g];
    const T c = kp.otfNorm[ch];
    const T* phf = kp.phiFixed + (size_t)ch * n2;
    for (int i = tid; i < Tile<N>::ELEMS; i += THREADS) s[i] = mkc<T>(0, 0);
    if (!kp.phiImg)
        for (int m = tid; m < kp.M; m += THREADS) al[m] = kp.alphaEff[g * kp.M + m];
    __syncthreads();
    for (int q = tid; q < n2; q += THREADS) {
        const T a = kp.A[q];
        cx<T> v = mkc<T>(0, 0);
        if (a > (T)0) {
            T sn, cs;
            sincos_t<T>(image_phase(kp, al, phf, g, q, n2), &sn, &cs);
            v = mkc<T>(a * cs, a * sn);
        }
        pf[q] = v;
        s[(q / n + n / 2) * LDS + q % n + n / 2] = cscale<T>(v, c);
    }
    __syncthreads();
}

// A scratch slot (one N x N tile of Xscr) for a block of a kernel that runs one work item per
// block: a free bit of the mask of the SM the block runs on.  An SM holds at most slotsPerSM
// blocks of these kernels at once (their occupancy, from which the slots were sized), so a
// free bit exists when a block starts; the bounded retries only absorb contention between
// blocks starting together.  A block that finds none records status 1 and skips its item
// (the host reports it).  Returns the slot or -1, in every thread.
__device__ __forceinline__ int acquire_slot(unsigned* masks, int perSM, int32_t* status, int* smidOut, int* bitOut) {
    __shared__ int slotSh, smidSh, bitSh;
    if (threadIdx.x == 0) {
        unsigned smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        const unsigned all = perSM >= 32 ? 0xffffffffu : ((1u << perSM) - 1u);
        int slot = -1, bit = -1;
        for (int tries = 0; tries < 256 && slot < 0; ++tries) {
            const unsigned freeBits = ~atomicOr(masks + smid, 0u) & all;
            if (!freeBits) continue;
            const int b = __ffs(freeBits) - 1;
            if (!(atomicOr(masks + smid, 1u << b) & (1u << b))) {
                slot = (int)smid * perSM + b;
                bit = b;
            }
        }
        if (slot < 0) atomicExch(status, 1);
        slotSh = slot;
        smidSh = (int)smid;
        bitSh = bit;
    }
    __syncthreads();
    *smidOut = smidSh;
    *bitOut = bitSh;
    return slotSh;
}
__device__ __forceinline__ void release_slot(unsigned* masks, int smid, int bit) {
    __syncthreads();    // every thread done with the slot
    if (threadIdx.x == 0 && bit >= 0) atomicAnd(masks + smid, ~(1u << bit));
}

// The adjoint with recomputed transforms, one image per block: PF -> X [-> S when SREC] ->
// G -> fft(G) X -> U -> projection; four transforms with SREC, three without (the general
// path keeps S, which its per-object accumulation reads).  (A persistent loop around the
// in-place transforms makes the compiler hoist their index arithmetic and spill.)
template <typename T, int N, int THREADS, bool SREC>
__global__ void __launch_bounds__(THREADS) k_adjoint_rc(KParams<T> kp, int kind) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    constexpr bool XS = PingPong<T, N>::value;            // X in a second shared tile
    constexpr int TILES = XS ? 2 : 1;
    static_assert(((size_t)(TILES * Tile<N>::ELEMS + N + n2) * sizeof(cx<T>)) % 16 == 0, "v is 16-byte aligned");
    const int nWork = *kp.nGradP * kp.I;
    const int w = blockIdx.x;
    if (w >= nWork) return;
    if (w % kp.I >= kp.pgeo[kp.gradP[w / kp.I]].nImg) return;   // an image slot the patch does not use
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* s = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* tw = s + TILES * Tile<N>::ELEMS;
    cx<T>* pf = tw + N;                            // [n2] pupil function
    T* v = reinterpret_cast<T*>(pf + n2);          // [n2] weights of the projection
    T* al = v + n2;                                // [M] coefficients
    int smid = -1, bit = -1;
    cx<T>* Xb;
    if constexpr (XS) {
        Xb = s + Tile<N>::ELEMS;
    } else {
        const int slot = acquire_slot(kp.slotMask, kp.slotsPerSM, kp.rcStatus, &smid, &bit);
        if (slot < 0) return;
        Xb = kp.Xscr + (size_t)slot * N2;
    }
    const int tid = (int)threadIdx.x;
    const T inv = (T)1 / (T)N2;
    const int p = kp.gradP[w / kp.I], j = w % kp.I;
    const size_t g = (size_t)p * kp.I + j;
    load_twiddles<T, N>(tw, kp.tw);
    recompute_pupil<T, N, THREADS>(kp, g, j, s, pf, al, tid);
    fft2d<T, N, -1, THREADS, true>(s, tw, tid);
    for (int i = tid; i < N2; i += THREADS) {
        const int y = i / N, x = i % N;
        const cx<T> X = s[y * LDS + x];
        Xb[i] = X;
        if (SREC) s[y * LDS + x] = mkc<T>(cnorm<T>(X), 0);
    }
    __syncthreads();
    if (SREC) fft2d<T, N, +1, THREADS, false>(s, tw, tid);
    const size_t po = (size_t)p * kp.nObj + kp.pImgObj[g];
    const cx<T>* Oo = kp.O + po * N2;
    const cx<T>* Dg = kp.D + g * N2;
    for (int i = tid; i < N2; i += THREADS) {
        const int y = i / N, x = i % N;                 // un-centred (lag) position
        const int c = ((y + N / 2) % N) * N + (x + N / 2) % N;
        const uint8_t m = kp.otfMask[c];
        const cx<T> O = Oo[c], D = Dg[c];
        const cx<T> S = SREC ? cscale<T>(s[y * LDS + x], inv) : kp.S[g * N2 + c];
        const cx<T> G = cmulc<T>(csub<T>(D, cmul<T>(O, S)), O);   // conj(O) (D - O S)
        s[y * LDS + x] = (m && !(y == 0 && x == 0)) ? G : mkc<T>(0, 0);
    }
    __syncthreads();
    fft2d<T, N, -1, THREADS, false>(s, tw, tid);
    for (int i = tid; i < N2; i += THREADS) {
        const int y = i / N, x = i % N;
        s[y * LDS + x] = cmul<T>(s[y * LDS + x], Xb[i]);
    }
    __syncthreads();
    fft2d_out_rows_pruned<T, N, +1, THREADS>(s, tw, tid);
    project_modes<T, N, THREADS>(kp, kind, p, j, s, pf, v, tid);
    if constexpr (!XS) release_slot(kp.slotMask, smid, bit);
}

// ----------------------------------------------------------------------------------
// Finite-difference gradient: SubImage::gradientFiniteDifference + metricChange
// (subimage.cpp:261-292), used by the reference for the first gradient of a patch.
// The OTF change dS = S(phi + h Z_m) - S(phi) is formed directly as
//     ifft(2 Re(conj(X) dX) + |dX|^2) / N^2,  dX = fft(c PF (exp(i h Z_m) - 1))
// instead of as a difference of two transforms, and metricChange is rearranged with
// G = conj(O)(D - O S) so that no large terms cancel:
//     dl = -sum [2 Q Re(dS conj G) + |dS|^2 (|D|^2 - Q |O|^2)] / (Q + dq) / N^2.
// One block per (image, mode).
// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS>
__device__ __forceinline__ void fd_image(const KParams<T>& kp, int p, int j, int m, const cx<T>* PF,
                                         const cx<T>* X, int tid) {
    const int g = p * kp.I + j;
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    constexpr bool PP = PingPong<T, N>::value;
    if (j >= kp.pgeo[p].nImg) return;   // an image slot the patch does not use
    const int o = kp.pImgObj[g];
    if (m >= kp.modeCount[p] || kp.objWeight[o] == 0.0) {
        if (tid == 0) kp.galpha[(size_t)g * kp.M + m] = 0.0;
        return;
    }
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* s = work_tile<T, N>(kp, smem_raw);
    cx<T>* s2 = s + (PP ? Tile<N>::ELEMS : 0);
    cx<T>* tw = GlobalTile<T, N>::value ? after_tile<T, N>(smem_raw) : s2 + Tile<N>::ELEMS;
    double* red = reinterpret_cast<double*>(tw + N);
    __syncthreads();    // previous item's shared memory consumed
    load_twiddles<T, N>(tw, kp.tw);
    for (int i = tid; i < Tile<N>::ELEMS; i += THREADS) s[i] = mkc<T>(0, 0);
    __syncthreads();
    const int ch = kp.pImgCh[g];
    const T c = kp.otfNorm[ch];
    const double h = kp.objGradStep[o];
    const T* Zm = kp.Z + (size_t)m * n2;
    for (int q = tid; q < n2; q += THREADS) {
        if (kp.A[q] > (T)0) {
            const T t = (T)h * Zm[q];
            T sh, ch2, sn, cs;
            sincos_t<T>(t * (T)0.5, &sh, &ch2);
            sincos_t<T>(t, &sn, &cs);
            const cx<T> e = mkc<T>((T)-2 * sh * sh, sn);   // exp(i t) - 1
            const int y = q / n, x = q % n;
            s[(y + n / 2) * LDS + x + n / 2] = cscale<T>(cmul<T>(PF[q], e), c);
        }
    }
    __syncthreads();
    if constexpr (PP) fft2d_pp<T, N, -1, THREADS, true>(s, s2, tw);
    else fft2d<T, N, -1, THREADS, true>(s, tw, tid);
    for (int i = tid; i < N2; i += THREADS) {
        const int y = i / N, x = i % N;
        const cx<T> dX = s[y * LDS + x];
        const cx<T> x0 = X[i];
        s[y * LDS + x] = mkc<T>((T)2 * (x0.x * dX.x + x0.y * dX.y) + cnorm<T>(dX), 0);
    }
    __syncthreads();
    if constexpr (PP) fft2d_pp<T, N, +1, THREADS, false>(s, s2, tw);
    else fft2d<T, N, +1, THREADS, false>(s, tw, tid);
    const size_t po = (size_t)p * kp.nObj + o;
    const T inv = (T)1 / (T)N2;
    double dl = 0;
    for (int i = tid; i < N2; i += THREADS) {
        if (!kp.otfMask[i]) continue;
        const int cy = i / N, cxx = i % N;
        if (cy == N / 2 && cxx == N / 2) continue;       // dS(0) = 0 exactly
        const int y = (cy + N / 2) % N, x = (cxx + N / 2) % N;
        const cx<T> dS = cscale<T>(s[y * LDS + x], inv);
        const cx<T> S = kp.S[(size_t)g * N2 + i];
        const cx<T> D = kp.D[(size_t)g * N2 + i];
        const cx<T> O = kp.O[po * N2 + i];
        const T Q = kp.Qt[po * N2 + i];
        const cx<T> G = cmulc<T>(csub<T>(D, cmul<T>(O, S)), O);
        const T dq = (T)2 * (S.x * dS.x + S.y * dS.y) + cnorm<T>(dS);
        const T num = (T)2 * Q * (dS.x * G.x + dS.y * G.y) + cnorm<T>(dS) * (cnorm<T>(D) - Q * cnorm<T>(O));
        dl -= (double)num / (double)(Q + dq);
    }
    const double tot = block_sum<THREADS>(dl, red);
    if (tid == 0) {
        const double w = kp.objWeight[o];
        kp.galpha[(size_t)g * kp.M + m] = w * (tot / (double)N2 / h * w);
    }
}

template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_fd(KParams<T> kp) {
    const int nWork = *kp.nFdP * kp.I * kp.M;
    auto item = [&](int w) {
        const int p = kp.fdP[w / (kp.M * kp.I)], j = (w / kp.M) % kp.I, m = w % kp.M;
        const size_t g = (size_t)p * kp.I + j;
        fd_image<T, N, THREADS>(kp, p, j, m, kp.PF + g * (N / 2) * (N / 2), kp.X + g * N * N, (int)threadIdx.x);
    };
    if constexpr (PingPong<T, N>::value || GlobalTile<T, N>::value) {
        // (a global work tile per block: the grid is the number of tiles)
        for (int w = blockIdx.x; w < nWork; w += gridDim.x) item(w);
    } else {
        const int w = blockIdx.x;
        if (w < nWork) item(w);
    }
}

// Shared memory of k_fd (and of k_fd_rc before its own arrays): tiles, twiddles, reduction.
template <typename T, int N>
constexpr size_t fd_base_smem() {
    return (size_t)((GlobalTile<T, N>::value ? 0 : PingPong<T, N>::value ? 2 : 1) * Tile<N>::ELEMS + N) * sizeof(cx<T>) +
           33 * sizeof(double);
}

// The finite-difference gradient with recomputed transforms.  FP32 up to N = 88 (ping-pong
// transforms, which a loop does not make spill): persistent, each block taking a contiguous
// range of (image, mode) items, modes fastest, and forming PF (shared memory) and X (its
// scratch slot, blockIdx.x) when its image changes.  Otherwise one (image, mode) item per
// block with X in a slot of its SM, formed for the item.
template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_fd_rc(KParams<T> kp) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n2 = (N / 2) * (N / 2), N2 = N * N;
    constexpr bool PP = PingPong<T, N>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* s = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* tw = s + (PP ? 2 : 1) * Tile<N>::ELEMS;
    cx<T>* pf = reinterpret_cast<cx<T>*>(smem_raw + ((fd_base_smem<T, N>() + 15) & ~(size_t)15));
    T* al = reinterpret_cast<T*>(pf + n2);
    const int nWork = *kp.nFdP * kp.I * kp.M;
    auto prepare = [&](size_t g, int j, cx<T>* Xb) {
        __syncthreads();    // the previous item's tiles consumed
        load_twiddles<T, N>(tw, kp.tw);
        recompute_pupil<T, N, THREADS>(kp, g, j, s, pf, al, (int)threadIdx.x);
        if constexpr (PP) fft2d_pp<T, N, -1, THREADS, true>(s, s + Tile<N>::ELEMS, tw);
        else fft2d<T, N, -1, THREADS, true>(s, tw, (int)threadIdx.x);
        for (int i = threadIdx.x; i < N2; i += THREADS) Xb[i] = s[(i / N) * LDS + i % N];
    };
    if constexpr (PP) {
        if ((int)blockIdx.x >= kp.scrBlocks) return;
        const int per = (nWork + (int)gridDim.x - 1) / (int)gridDim.x;
        const int w0 = (int)blockIdx.x * per, w1 = min(nWork, w0 + per);
        cx<T>* Xb = kp.Xscr + (size_t)blockIdx.x * N2;
        long gPrev = -1;
        for (int w = w0; w < w1; ++w) {
            const int p = kp.fdP[w / (kp.M * kp.I)], j = (w / kp.M) % kp.I, m = w % kp.M;
            const size_t g = (size_t)p * kp.I + j;
            if (j < kp.pgeo[p].nImg && m < kp.modeCount[p] && kp.objWeight[kp.pImgObj[g]] != 0.0 &&
                (long)g != gPrev) {
                prepare(g, j, Xb);
                gPrev = (long)g;
            }
            fd_image<T, N, THREADS>(kp, p, j, m, pf, Xb, (int)threadIdx.x);
        }
    } else {
        const int w = blockIdx.x;
        if (w >= nWork) return;
        const int p = kp.fdP[w / (kp.M * kp.I)], j = (w / kp.M) % kp.I, m = w % kp.M;
        const size_t g = (size_t)p * kp.I + j;
        if (j >= kp.pgeo[p].nImg) return;   // an image slot the patch does not use
        if (m >= kp.modeCount[p] || kp.objWeight[kp.pImgObj[g]] == 0.0) {
            if (threadIdx.x == 0) kp.galpha[g * kp.M + m] = 0.0;
            return;
        }
        int smid = -1, bit = -1;
        const int slot = acquire_slot(kp.slotMask, kp.slotsPerSM, kp.rcStatus, &smid, &bit);
        if (slot < 0) return;
        cx<T>* Xb = kp.Xscr + (size_t)slot * N2;
        prepare(g, j, Xb);
        fd_image<T, N, THREADS>(kp, p, j, m, pf, Xb, (int)threadIdx.x);
        release_slot(kp.slotMask, smid, bit);
    }
}

}  // namespace rdxg
