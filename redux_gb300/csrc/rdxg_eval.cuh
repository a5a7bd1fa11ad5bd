// Fused metric evaluation (FP32 path): forward model + per-object accumulation in one pass.
//
// The reference forms every image's OTF, accumulates P = sum conj(D) S and Q = gamma +
// sum |S|^2 per object and sums |D|^2 - |P|^2/Q over the OTF support
// (Solver::metric, solver.cpp:763-817; Object::addToPQ/calcMetric, object.cpp:508-615).
// Here one thread block takes a chunk of an object's images; for each image it builds the
// OTF in shared memory and immediately folds it into per-frequency accumulators held in
// registers, relative to a reference object O' of the same patch:
//     R  += |D - O' S|^2,   P' += conj(D - O' S) S,   Q += |S|^2.
// For any O' the object's term is exactly
//     sum_u  R + gamma |O'|^2 - |conj(P') - gamma O'|^2 / (gamma + Q),
// and it is free of cancellation when O' is close to conj(P)/Q.  O' is refreshed from every
// gradient evaluation (O = O' + (conj(P') - gamma O') / Q, exact) and by one extra pass
// after image re-initialisation.  D, S and O' are Hermitian (real images and PSFs), so only
// the half of the OTF support with (cy > N/2) or (cy == N/2 and cx >= N/2) is accumulated,
// the other half counting through a weight of 2 (1 for the DC term).
// The OTF is written to HBM only for gradient evaluations, which need it again.
// Measured against the FP64 oracle with O' taken at the last gradient point and steps along
// the gradient, pure tilt and random directions, the metric agrees to 1e-8 ... 3e-7, the
// same as with O' taken at the evaluated point (FP32 accumulation is enough).
#pragma once

#include "rdxg_kernels.cuh"

namespace rdxg {

struct EvalItem {
    int32_t p, o, first, count, chunk, df;
};

struct PoItem {
    int32_t p, o, mode;   // mode: 0 metric, 1 gradient (write O, Qt), 2 refresh O'
};

struct Lists {
    EvalItem* eval;  int32_t* nEval;
    PoItem* po;      int32_t* nPo;
    int32_t* gradP;  int32_t* nGradP;   // patches that need the analytic gradient
    int32_t* fdP;    int32_t* nFdP;     // patches that need the finite-difference gradient
    int32_t* counters;                  // base of the counters (reset every round)
};

struct HalfPlane {
    int32_t nH;
    const int32_t* idx;     // [nH] centred index of each half-plane support point
    int32_t chunkSize;      // images per chunk
    int32_t chunksPerPatch; // sum over objects of ceil(count / chunkSize)
    const int32_t* objChunk0;  // [nObj] first chunk of each object within a patch
};

template <typename T>
struct EvalParams {
    KParams<T> k;
    HalfPlane hp;
    const cx<T>* Dh;    // [g][nH] half-plane image transforms
    cx<T>* Oh;          // [po][nH] reference objects
    T* part;            // [P*chunksPerPatch][4][nH]  (R, Q, P're, P'im)
    double* objMetric;  // [po][tiles] per-tile partial sums of the object metric
    const int32_t* hPos; // [nH] tile position (row * (N+1) + column) of each half-plane point
    int32_t nTilesH;    // point tiles per object in the reduction
    T* phi;             // [g][n*n] phases of the images being evaluated (k_phase)
    Lists L;
};

// ----------------------------------------------------------------------------------
// Mode expansion for every image of the work list: phi = phi_fixed + sum_m alpha_m Z_m
// (SubImage::calcPhi / addToPhi, subimage.cpp:509-544) as a small GEMM
// [images x M] x [M x n*n].  One block per (chunk, tile of PIX pixels): the modes of the
// tile are staged in shared memory once and each thread accumulates its pixel for all
// images of the chunk.
// ----------------------------------------------------------------------------------
template <typename T, int N, int PIX, int MAXC>
__global__ void __launch_bounds__(PIX) k_phase(EvalParams<T> e) {
    constexpr int n2 = (N / 2) * (N / 2);
    constexpr int nPix = (n2 + PIX - 1) / PIX;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = e.k.M;
    T* zs = reinterpret_cast<T*>(smem_raw);          // [M][PIX]
    T* as = zs + (size_t)M * PIX;                    // [MAXC][M]
    const int nWork = *e.L.nEval * nPix;
    for (int w = blockIdx.x; w < nWork; w += gridDim.x) {
        const EvalItem it = e.L.eval[w / nPix];
        const int q0 = (w % nPix) * PIX;
        const int q = q0 + threadIdx.x;
        __syncthreads();
        for (int i = threadIdx.x; i < M * PIX; i += PIX) {
            const int m = i / PIX, qq = q0 + i % PIX;
            zs[i] = qq < n2 ? e.k.Z[(size_t)m * n2 + qq] : (T)0;
        }
        const size_t g0 = (size_t)it.p * e.k.I + it.first;
        for (int i = threadIdx.x; i < it.count * M; i += PIX) as[i] = e.k.alphaEff[g0 * M + i];
        __syncthreads();
        if (q >= n2) continue;
        T acc[MAXC];
#pragma unroll
        for (int c = 0; c < MAXC; ++c) acc[c] = (T)0;
        for (int m = 0; m < M; ++m) {
            const T z = zs[m * PIX + threadIdx.x];
#pragma unroll
            for (int c = 0; c < MAXC; ++c) acc[c] += as[c * M + m] * z;
        }
        for (int c = 0; c < it.count && c < MAXC; ++c) {
            const int j = it.first + c;
            e.phi[(g0 + c) * n2 + q] = e.k.phiFixed[(size_t)e.k.imgCh[j] * n2 + q] + acc[c];
        }
    }
}

// One image of a chunk: forward model in the shared tile (transforms ping-pong between s
// and s2), then the accumulation.
template <typename T, int N, int THREADS>
__device__ __forceinline__ void eval_image(const T* __restrict__ phi_g, const T* __restrict__ A, T c, int df,
                                           cx<T>* PF, cx<T>* X, cx<T>* S, const cx<T>* __restrict__ Dg,
                                           cx<T>* s, cx<T>* s2, const cx<T>* tw, const cx<T>* oh,
                                           T* acc, const int* hpos, int nH) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    const T inv = (T)1 / (T)N2;
    __syncthreads();    // previous image's tile fully consumed
    zero_tile<T, N>(s);
    __syncthreads();
    for (int q = threadIdx.x; q < n2; q += THREADS) {
        const T a = A[q];
        cx<T> pf = mkc<T>(0, 0);
        if (a > (T)0) {
            T sn, cs;
            sincos_t<T>(phi_g[q], &sn, &cs);
            pf = mkc<T>(a * cs, a * sn);
        }
        if (df) PF[q] = pf;
        const int y = q / n, x = q % n;
        s[(y + n / 2) * LDS + x + n / 2] = cscale<T>(pf, c);
    }
    __syncthreads();
    fft2d_pp<T, N, -1, THREADS, true>(s, s2, tw);
    for (int i = threadIdx.x; i < N2; i += THREADS) {
        const int y = i / N, x = i % N;
        const cx<T> v = s[y * LDS + x];
        if (df) X[i] = v;
        s[y * LDS + x] = mkc<T>(cnorm<T>(v), 0);
    }
    __syncthreads();
    fft2d_pp<T, N, +1, THREADS, false>(s, s2, tw);
    if (df) {
        for (int i = threadIdx.x; i < N2; i += THREADS) {
            const int cy = i / N, cxx = i % N;
            const int y = (cy + N / 2) % N, x = (cxx + N / 2) % N;
            S[i] = cscale<T>(s[y * LDS + x], inv);
        }
    }
    for (int h = threadIdx.x; h < nH; h += THREADS) {
        const cx<T> sv = cscale<T>(s[hpos[h]], inv);
        const cx<T> r = csub<T>(Dg[h], cmul<T>(oh[h], sv));
        // R += |r|^2, Q += |S|^2, P' += conj(r) S
        acc[h] += cnorm<T>(r);
        acc[nH + h] += cnorm<T>(sv);
        acc[2 * nH + h] += r.x * sv.x + r.y * sv.y;
        acc[3 * nH + h] += r.x * sv.y - r.y * sv.x;
    }
}

// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS, int NPT>
__global__ void __launch_bounds__(THREADS, 1) k_eval(EvalParams<T> e) {
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nH = e.hp.nH;
    // shared memory: two tiles | twiddles | reference object | accumulators (4 x nH) |
    //                tile positions
    cx<T>* s = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s2 = s + Tile<N>::ELEMS;
    cx<T>* tw = s2 + Tile<N>::ELEMS;
    cx<T>* oh = tw + N;
    T* acc = reinterpret_cast<T*>(oh + nH);
    int* hpos = reinterpret_cast<int*>(acc + 4 * nH);
    load_twiddles<T, N>(tw, e.k.tw);
    for (int h = threadIdx.x; h < nH; h += THREADS) hpos[h] = e.hPos[h];
    const int nItems = *e.L.nEval;
    for (int item = blockIdx.x; item < nItems; item += gridDim.x) {
        const EvalItem it = e.L.eval[item];
        const size_t po = (size_t)it.p * e.k.nObj + it.o;
        __syncthreads();    // previous item's accumulators written out
        for (int h = threadIdx.x; h < nH; h += THREADS) oh[h] = e.Oh[po * nH + h];
        for (int i = threadIdx.x; i < 4 * nH; i += THREADS) acc[i] = (T)0;
        for (int jj = 0; jj < it.count; ++jj) {
            const int j = it.first + jj;
            const size_t g = (size_t)it.p * e.k.I + j;
            const int ch = e.k.imgCh[j];
            eval_image<T, N, THREADS>(e.phi + g * n2, e.k.A, e.k.otfNorm[ch], it.df, e.k.PF + g * n2,
                                      e.k.X + g * N2, e.k.S + g * N2, e.Dh + g * nH, s, s2, tw, oh, acc, hpos, nH);
        }
        __syncthreads();
        T* part = e.part + (size_t)(it.p * e.hp.chunksPerPatch + it.chunk) * 4 * nH;
        for (int i = threadIdx.x; i < 4 * nH; i += THREADS) part[i] = acc[i];
    }
}

// ----------------------------------------------------------------------------------
// Per-object reduction over the chunks (fixed order) and the object metric: one block per
// (object, tile of points); the per-tile partial sums (double) are added in a fixed order by
// the solver.  mode 1 (gradient) and 2 (refresh) replace O' by the exact object O of this
// point; mode 1 also writes O and Q on the full plane for the gradient kernels.
// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_reduce(EvalParams<T> e) {
    __shared__ double red[33];
    const int nItems = *e.L.nPo * e.nTilesH;
    const int nH = e.hp.nH;
    for (int w = blockIdx.x; w < nItems; w += gridDim.x) {
        const PoItem it = e.L.po[w / e.nTilesH];
        const int tile = w % e.nTilesH;
        const size_t po = (size_t)it.p * e.k.nObj + it.o;
        const T gam = (T)e.k.gamma[po];
        const int c0 = e.hp.objChunk0[it.o];
        const int nc = (e.k.objCount[it.o] + e.hp.chunkSize - 1) / e.hp.chunkSize;
        const T* base = e.part + (size_t)(it.p * e.hp.chunksPerPatch + c0) * 4 * nH;
        double acc = 0;
        const int h = tile * THREADS + threadIdx.x;
        if (h < nH) {
            T R = 0, Q = 0, Pr = 0, Pi = 0;
            for (int c = 0; c < nc; ++c) {
                const T* pc = base + (size_t)c * 4 * nH + h;
                R += pc[0]; Q += pc[nH]; Pr += pc[2 * nH]; Pi += pc[3 * nH];
            }
            const cx<T> oh = e.Oh[po * nH + h];
            const T Qt = gam + Q;
            // conj(P') - gamma O'
            const T dPr = Pr - gam * oh.x, dPi = -Pi - gam * oh.y;
            const T term = R + gam * cnorm<T>(oh) - (dPr * dPr + dPi * dPi) / Qt;
            const int cidx = e.hp.idx[h];
            const bool dc = (cidx == (N / 2) * N + N / 2);
            acc = dc ? (double)term : 2.0 * (double)term;
            if (it.mode != 0) {
                const cx<T> O = mkc<T>(oh.x + dPr / Qt, oh.y + dPi / Qt);
                e.Oh[po * nH + h] = O;
                if (it.mode == 1) {
                    const int cy = cidx / N, cxx = cidx % N;
                    const int partner = ((N - cy) % N) * N + (N - cxx) % N;
                    e.k.O[po * N * N + cidx] = O;
                    e.k.Qt[po * N * N + cidx] = Qt;
                    e.k.O[po * N * N + partner] = mkc<T>(O.x, -O.y);
                    e.k.Qt[po * N * N + partner] = Qt;
                }
            }
        }
        const double tot = block_sum<THREADS>(acc, red);
        if (threadIdx.x == 0) e.objMetric[po * e.nTilesH + tile] = tot;
    }
}

}  // namespace rdxg
