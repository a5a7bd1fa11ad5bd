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
// the half of the OTF support with (cx > N/2) or (cx == N/2 and cy >= N/2) is accumulated,
// the other half counting through a weight of 2 (1 for the DC term).
// The OTF is written to HBM only for gradient evaluations, which need it again.
// Measured against the FP64 oracle with O' taken at the last gradient point and steps along
// the gradient, pure tilt and random directions, the metric agrees to 1e-8 ... 3e-7, the
// same as with O' taken at the evaluated point (FP32 accumulation is enough).
#pragma once

#include <cuda_bf16.h>

#include "rdxg_kernels.cuh"

namespace rdxg {

struct EvalItem {
    int32_t p, o, first, count, chunk, df;
};

struct PoItem {
    int32_t p, o, mode;   // mode: 0 metric, 1 gradient (write O, Qt), 2 refresh O'
};

// Half-plane points the fused evaluation takes at most: the half plane, capped at 3584 (seven
// accumulator records per thread of a 512-thread block, in registers).  A circular pupil's
// OTF support has about 0.42 N^2 of them (3237 at N = 88).
template <int N> struct kFusedMaxPoints {
    static constexpr int half = N * (N / 2 + 1);
    static constexpr int value = half < 3584 ? half : 3584;
};

// half-plane points per work item of the object reduction (k_reduce): four per lane
constexpr int kReduceTile = 128;

// work-list counters (reset every round); the evaluation's claim and finished-block counters
// are reset by the evaluation itself (its last block), so that it can be launched again on the
// same lists
enum : int32_t { kCounterEval = 0, kCounterPo = 1, kCounterGrad = 2, kCounterFd = 3, kCounterEvalP = 4,
                 kCounterShift = 5, kCounterEvalClaim = 6, kCounterEvalDone = 7, kCounterCgDone = 8 };

struct Lists {
    EvalItem* eval;  int32_t* nEval;
    PoItem* po;      int32_t* nPo;
    int32_t* gradP;  int32_t* nGradP;   // patches that need the analytic gradient
    int32_t* fdP;    int32_t* nFdP;     // patches that need the finite-difference gradient
    int32_t* evalP;  int32_t* nEvalP;   // patches with an evaluation this round
    int32_t* counters;                  // base of the counters (reset every round)
};

// Per half-plane point sums of a chunk: R = sum |D - O'S|^2, Q = sum |S|^2, P' = sum conj(D - O'S) S,
// one 16-byte record per point (one vector load and store per update)
template <typename T> struct alignas(4 * sizeof(T)) Acc4 { T r, q, pr, pi; };

struct HalfPlane {
    int32_t nH;
    const int32_t* idx;     // [nH] centred index of each half-plane support point
    int32_t chunkSize;      // images per chunk
    int32_t chunksPerPatch; // sum over objects of ceil(count / chunkSize)
    const int32_t* objChunk0;  // [P][nObj] first chunk of each object within its patch
};

// Mode expansion on the tensor cores (rdxg_phase_tc.cu): the launch shape chosen per job.
struct PhaseTcPlan {
    int32_t valid, ntmax, G, NT, KP, parts, nTiles, grid;   // G patches (G*I images) per column tile
    int32_t occ;                                             // resident blocks per SM (occupancy query)
    size_t smem, zElems;                                     // dynamic shared memory; split mode elements
};

struct PhaseTcArgs {
    const __nv_bfloat16* Zt;   // [tile][part][128 x KP] split modes in the operand layout
    const float* alphaEff;     // [g][M]
    const float* phiFixed;     // [C][n*n]
    const int32_t* imgCh;      // [P][I] channel of each image slot of each patch
    const int32_t* evalP;      // patches with an evaluation this round
    const int32_t* nEvalP;
    float* phi;                // [g][n*n]
    int32_t* status;           // non-zero once a wait on the tensor core or copy engine gave up
    int32_t I, M, n2, nCh, G, NT, KP, parts;
};

template <typename T>
struct EvalParams {
    KParams<T> k;
    HalfPlane hp;
    const cx<T>* Dh;    // [g][nH] half-plane image transforms
    cx<T>* Oh;          // [po][nH] reference objects
    Acc4<T>* part;      // [P*chunksPerPatch][nH] (R, Q, P're, P'im)
    double* objMetric;  // [po][tiles] object metric summed over tiles of 32 half-plane points
    const int32_t* hPos; // [nH] tile position (row * (N+1) + column) of each half-plane point
    int32_t nTilesH;    // point tiles (kReduceTile points) per object in the reduction
    T* phi;             // [g][n*n] phases of the images being evaluated (k_phase)
    int32_t nCh;        // channels (fixed phases)
    Lists L;
    const __nv_bfloat16* Zt;   // split modes of the tensor-core mode expansion (null: CUDA cores)
    int32_t* tcStatus;
    PhaseTcPlan tc;
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
            e.phi[(g0 + c) * n2 + q] = e.k.phiFixed[(size_t)e.k.pImgCh[g0 + c] * n2 + q] + acc[c];
        }
    }
}

// Asynchronous 8-byte global -> shared copies (cp.async): the phases of the next image and
// the transforms of the current one are fetched into parts of the two tiles that the
// transforms leave unused at that time, so no thread waits on global memory.
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Mode expansion per patch with the modes in registers.  The grid is a multiple of the
// number of pixel tiles: block b always takes pixel tile b % nPix (its thread holds Z_m at
// its pixel for m < MAXM in registers, zero beyond M) and walks the patches to evaluate
// with stride gridDim.x / nPix.  A patch's coefficients are one contiguous block
// alphaEff[p*I .. p*I + I) x M; the next patch's block is copied into the other of two
// shared buffers (cp.async) while the current one is expanded, four images at a time (four
// independent sums, coefficients read four modes at a time).  Each sum runs over m in
// order, then the fixed phase of the image's channel is added, as in k_phase.
template <typename T, int N, int PIX, int MAXM, int MAXI, int MAXCH>
__global__ void __launch_bounds__(PIX, 4) k_phase_patch(EvalParams<T> e) {
    constexpr int n2 = (N / 2) * (N / 2);
    constexpr int nPix = (n2 + PIX - 1) / PIX;
    static_assert(MAXM % 4 == 0 && MAXI % 4 == 0, "modes and images go four at a time");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* as = reinterpret_cast<T*>(smem_raw);          // [2][MAXI][MAXM]
    T* pfs = as + 2 * MAXI * MAXM;                   // [MAXCH][PIX]
    int* chs = reinterpret_cast<int*>(pfs + MAXCH * PIX);   // [2][MAXI]
    const int M = e.k.M, I = e.k.I;
    const int nP = *e.L.nEvalP;
    const int S = gridDim.x / nPix;
    const int s0 = blockIdx.x / nPix;
    if (s0 >= nP) return;
    const int q0 = (blockIdx.x % nPix) * PIX;
    const int q = q0 + threadIdx.x;
    T z[MAXM];
#pragma unroll
    for (int m = 0; m < MAXM; ++m) z[m] = (m < M && q < n2) ? e.k.Z[(size_t)m * n2 + q] : (T)0;
    // zero both buffers once: the copies only fill m < M of rows < I
    for (int i = threadIdx.x; i < 2 * MAXI * MAXM; i += PIX) as[i] = (T)0;
    for (int i = threadIdx.x; i < e.nCh * PIX; i += PIX) {
        const int qq = q0 + i % PIX;
        pfs[i] = qq < n2 ? e.k.phiFixed[(size_t)(i / PIX) * n2 + qq] : (T)0;
    }
    __syncthreads();
    const int IM = I * M;
    auto fetch = [&](int k, int buf) {
        const int p = e.L.evalP[k];
        const T* src = e.k.alphaEff + (size_t)p * IM;
        T* dst = as + buf * MAXI * MAXM;
        for (int i = threadIdx.x; i < IM; i += PIX) cp_async4(dst + (i / M) * MAXM + i % M, src + i);
        // the channel of each image slot of the patch (two buffers, like the coefficients)
        for (int i = threadIdx.x; i < MAXI; i += PIX) chs[buf * MAXI + i] = i < I ? e.k.pImgCh[(size_t)p * I + i] : 0;
    };
    fetch(s0, 0);
    cp_async_commit();
    int buf = 0;
    for (int k = s0; k < nP; k += S) {
        if (k + S < nP) fetch(k + S, buf ^ 1);
        cp_async_commit();
        cp_async_wait_one();
        __syncthreads();
        if (q < n2) {
            const int p = e.L.evalP[k];
            const T* ab = as + buf * MAXI * MAXM;
            for (int i = 0; i < I; i += 4) {
                const T* al = ab + i * MAXM;
                T acc0 = (T)0, acc1 = (T)0, acc2 = (T)0, acc3 = (T)0;
#pragma unroll
                for (int m = 0; m < MAXM; m += 4) {
                    const float4 a0 = *reinterpret_cast<const float4*>(al + m);
                    const float4 a1 = *reinterpret_cast<const float4*>(al + MAXM + m);
                    const float4 a2 = *reinterpret_cast<const float4*>(al + 2 * MAXM + m);
                    const float4 a3 = *reinterpret_cast<const float4*>(al + 3 * MAXM + m);
                    acc0 += a0.x * z[m]; acc0 += a0.y * z[m + 1]; acc0 += a0.z * z[m + 2]; acc0 += a0.w * z[m + 3];
                    acc1 += a1.x * z[m]; acc1 += a1.y * z[m + 1]; acc1 += a1.z * z[m + 2]; acc1 += a1.w * z[m + 3];
                    acc2 += a2.x * z[m]; acc2 += a2.y * z[m + 1]; acc2 += a2.z * z[m + 2]; acc2 += a2.w * z[m + 3];
                    acc3 += a3.x * z[m]; acc3 += a3.y * z[m + 1]; acc3 += a3.z * z[m + 2]; acc3 += a3.w * z[m + 3];
                }
                const T accs[4] = {acc0, acc1, acc2, acc3};
                T* out = e.phi + ((size_t)p * I + i) * n2 + q;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (i + j < I) out[(size_t)j * n2] = pfs[chs[buf * MAXI + i + j] * PIX + threadIdx.x] + accs[j];
            }
        }
        __syncthreads();    // buffer fully read before the next copy into it
        buf ^= 1;
    }
    cp_async_wait_all();
}

// Staging places of the image transforms Dh (W = N/2 + 1 slots per tile row; the columns
// [N/2, N] of the rows [N/2, N) of both tiles are left alone by the half-plane core after
// its first column stage): h < N/2 * W in tile a, the rest in tile b.
template <int N> struct Stage {
    static constexpr int LDS = N + 1, W = N / 2 + 1;
    static constexpr int kPart = (N / 2) * W;     // points per tile
    static constexpr int kMaxH = 2 * kPart;
    static __device__ __forceinline__ int dh_slot(int h) {   // within its tile
        const int k = h < kPart ? h : h - kPart;
        return (N / 2 + k / W) * LDS + N / 2 + k % W;
    }
};

template <typename T, int N, int THREADS>
__device__ __forceinline__ void stage_phi(T* buf, const T* __restrict__ phi_g) {
    constexpr int pairs = (N / 2) * (N / 2) / 2;
    for (int p = threadIdx.x; p < pairs; p += THREADS) cp_async8(buf + 2 * p, phi_g + 2 * p);
}

// Half-plane OTF core.  On entry tile a holds the pupil-plane field at rows and columns
// [N/4, 3N/4) (the caller embeds it there); the first stage of the row pass loads only those
// columns of those rows.  The column pass loads only those rows in its first stage;
// its last stage hands every transform value v at (row e, column x) to elem(e, x, v), which
// returns a real value (|X|^2 for the OTF) stored as the real (e even) or imaginary (e odd)
// part of row e/2 of tile a: two real rows packed as one complex row.  The N/2 packed rows are
// inverse-transformed along x; the first stage along y splits them again as it loads
// (A = (Z(k) + conj Z(-k))/2, B = (Z(k) - conj Z(-k))/2i) and only the columns [0, N/2),
// which hold the half-plane points, are transformed along y.  On return tile a holds N^2
// times the inverse transform in those columns.  afterRows, afterCols1, afterPack run after
// the row pass, the first column stage and the packing stage (where the caller issues copies
// into the free parts of the tiles); midColumns runs between the two stages along y.
template <typename T, int N, int THREADS, typename PL = Plan<N>, typename Elem, typename HR, typename HC,
          typename HP, typename HM>
__device__ __forceinline__ void half_plane_core(cx<T>* a, cx<T>* b, const cx<T>* tw, Elem elem, HR afterRows,
                                                HC afterCols1, HP afterPack, HM midColumns) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int R1 = PL::R1, R2 = PL::R2;
    constexpr int LO = R1 / 4, HI = 3 * R1 / 4;      // non-zero inputs of the pruned first stage
    static_assert(R1 % 4 == 0, "the pruned first stage needs a radix divisible by 4");
    T* af = reinterpret_cast<T*>(a);
    // rows [N/4, 3N/4): the pupil field -> b -> a
    fft_stage_pp<T, N, R1, 1, -1, N / 2, THREADS, LO, HI>(a, b, N / 4, LDS, 1, tw);
    afterRows();
    fft_stage_pp<T, N, R2, R1, -1, N / 2, THREADS>(b, a, N / 4, LDS, 1, tw);
    // all columns (a -> b), then the last stage into the packed rows of a
    fft_stage_pp<T, N, R1, 1, -1, N, THREADS, LO, HI>(a, b, 0, 1, LDS, tw);
    afterCols1();
    fft_stage_fn<T, N, R2, R1, -1, N, THREADS, 0, R2>(
        0, tw, [&](int x, int e) { return b[e * LDS + x]; },
        [&](int x, int e, cx<T> v) { af[(e >> 1) * 2 * LDS + 2 * x + (e & 1)] = elem(e, x, v); });
    afterPack();
    // inverse along x on the N/2 packed rows (a -> b -> a)
    fft_stage_pp<T, N, R1, 1, +1, N / 2, THREADS>(a, b, 0, LDS, 1, tw);
    fft_stage_pp<T, N, R2, R1, +1, N / 2, THREADS>(b, a, 0, LDS, 1, tw);
    // inverse along y on the columns [0, N/2), splitting the packed rows as they are loaded
    fft_stage_fn<T, N, R1, 1, +1, N / 2, THREADS, 0, R1>(
        0, tw,
        [&](int k, int e) {
            const cx<T> z = a[(e >> 1) * LDS + k];
            const cx<T> zc = a[(e >> 1) * LDS + ((N - k) % N)];
            return (e & 1) ? mkc<T>((T)0.5 * (z.y + zc.y), (T)0.5 * (zc.x - z.x))    // (z - conj zc)/2i
                           : mkc<T>((T)0.5 * (z.x + zc.x), (T)0.5 * (z.y - zc.y));   // (z + conj zc)/2
        },
        [&](int k, int e, cx<T> v) { b[e * LDS + k] = v; });
    midColumns();
    fft_stage_pp<T, N, R2, R1, +1, N / 2, THREADS>(b, a, 0, 1, LDS, tw);
}

// Arithmetic of the evaluation written with explicitly rounded operations, so that the
// compiler has no choice of contraction left: every form of the kernel that uses these
// helpers forms the same bits.
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// c PF at a pupil pixel of amplitude amp and phase ph; the pupil function itself in *pf
template <typename T>
__device__ __forceinline__ cx<T> pupil_field(T amp, T ph, T c, cx<T>* pf) {
    cx<T> v = mkc<T>(0, 0);
    if (amp > (T)0) {
        T sn, cs;
        sincos_t<T>(ph, &sn, &cs);
        v = mkc<T>(mul_rn(amp, cs), mul_rn(amp, sn));
    }
    *pf = v;
    return mkc<T>(mul_rn(v.x, c), mul_rn(v.y, c));
}

// One half-plane point of a chunk's sums: s = N^2 S (the transform's output), d = D, o = O'
//     R += |D - O'S|^2,  Q += |S|^2,  P' += conj(D - O'S) S
template <typename T>
__device__ __forceinline__ void acc_point(Acc4<T>& u, cx<T> d, cx<T> o, cx<T> s, T inv) {
    const T sx = mul_rn(s.x, inv), sy = mul_rn(s.y, inv);
    const T osr = fma_rn(o.x, sx, -mul_rn(o.y, sy));
    const T osi = fma_rn(o.x, sy, mul_rn(o.y, sx));
    const T rx = add_rn(d.x, -osr), ry = add_rn(d.y, -osi);
    u.r = add_rn(u.r, fma_rn(rx, rx, mul_rn(ry, ry)));
    u.q = add_rn(u.q, fma_rn(sx, sx, mul_rn(sy, sy)));
    u.pr = add_rn(u.pr, fma_rn(rx, sx, mul_rn(ry, sy)));
    u.pi = add_rn(u.pi, fma_rn(rx, sy, -mul_rn(ry, sx)));
}

// One image of a chunk: the OTF on the half plane (half_plane_core with elem = |X|^2),
// folded into the chunk's accumulators, which live in registers: thread t holds the records of
// the points t + i * THREADS.  On entry the phases of this image are in phiBuf; phiNext (or
// null) is the next image's, fetched into phiBuf once the row pass has read it.
template <typename T, int N, int THREADS, int ACC, typename PL = Plan<N>>
__device__ __forceinline__ void eval_image(const T* __restrict__ phiNext, T* phiBuf, const T* A, T c, int keepPX,
                                           int keepS,
                                           cx<T>* PF, cx<T>* X, cx<T>* S, const cx<T>* __restrict__ Dg,
                                           cx<T>* a, cx<T>* b, const cx<T>* tw, const cx<T>* oh,
                                           Acc4<T> (&acc)[ACC], const uint16_t* hpos, const int* hidx, int nH) {
    constexpr int n = N / 2, N2 = N * N;
    static_assert(sizeof(cx<T>) == 8, "staging copies 8-byte elements");
    using St = Stage<N>;
    const T inv = (T)1 / (T)N2;
    __syncthreads();    // previous image's tiles fully consumed, staged phases visible
    const int nFirst = nH < St::kPart ? nH : St::kPart;
    // c PF of every pupil pixel first, in one balanced pass, into its embedded place in tile a
    // (rows and columns [N/4, 3N/4), where the first row stage reads it)
#pragma unroll 1
    for (int q = threadIdx.x; q < n * n; q += THREADS) {
        cx<T> pf;
        const cx<T> v = pupil_field<T>(A[q], phiBuf[q], c, &pf);
        if (keepPX) PF[q] = pf;
        a[(q / n + N / 4) * Tile<N>::LDS + q % n + N / 4] = v;
    }
    __syncthreads();
    auto elem = [&](int e, int x, cx<T> v) {
        if (keepPX) X[e * N + x] = v;
        return cnorm<T>(v);
    };
    auto afterRows = [&] {
        if (phiNext) stage_phi<T, N, THREADS>(phiBuf, phiNext);
        cp_async_commit();
    };
    auto afterCols1 = [&] {
        for (int h = threadIdx.x; h < nFirst; h += THREADS) cp_async8(a + St::dh_slot(h), Dg + h);
        cp_async_commit();
    };
    auto afterPack = [&] {
        for (int h = nFirst + threadIdx.x; h < nH; h += THREADS) cp_async8(b + St::dh_slot(h), Dg + h);
        cp_async_commit();
    };
    auto midColumns = [&] { cp_async_wait_all(); };
    half_plane_core<T, N, THREADS, PL>(a, b, tw, elem, afterRows, afterCols1, afterPack, midColumns);
    if (keepS) {
        // the full OTF from the half plane (S(-u) = conj S(u)) for the gradient kernels
        for (int h = threadIdx.x; h < nH; h += THREADS) {
            const cx<T> v = cscale<T>(a[hpos[h]], inv);
            const int cidx = hidx[h];
            const int cy = cidx / N, cxx = cidx % N;
            S[cidx] = v;
            S[((N - cy) % N) * N + (N - cxx) % N] = mkc<T>(v.x, -v.y);
        }
    }
#pragma unroll
    for (int i = 0; i < ACC; ++i) {
        const int h = (int)threadIdx.x + i * THREADS;
        if (h < nH) {
            const cx<T> d = (h < St::kPart ? a : b)[St::dh_slot(h)];
            acc_point<T>(acc[i], d, oh[h], a[hpos[h]], inv);
        }
    }
}

// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS, int NPT, typename PL = Plan<N>>
__global__ void __launch_bounds__(THREADS, 1) k_eval(EvalParams<T> e) {
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int nH = e.hp.nH;
    // shared memory: two tiles | twiddles | reference object | pupil amplitude | phases of
    //                the image | tile positions (16-bit)
    cx<T>* s = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s2 = s + Tile<N>::ELEMS;
    cx<T>* tw = s2 + Tile<N>::ELEMS;
    cx<T>* oh = tw + N;
    // the chunk's accumulators (R, Q, P') of the points threadIdx.x + i * THREADS
    constexpr int ACC = (kFusedMaxPoints<N>::value + THREADS - 1) / THREADS;
    Acc4<T> acc[ACC];
    T* amp = reinterpret_cast<T*>(oh + nH);
    T* phiBuf = amp + n2;
    uint16_t* hpos = reinterpret_cast<uint16_t*>(phiBuf + n2);
    static_assert(Tile<N>::ELEMS <= 65536, "tile positions are 16-bit");
    const int nItems = *e.L.nEval;
    // Work items: the block's first two by block index, then claimed from a counter one item
    // ahead (so the claim's latency is hidden behind a whole item), so that blocks that start
    // late (the SMs busy with another handle's kernels) take fewer items.  Each item's sums are
    // the same whichever block forms them.
    __shared__ int claimSh;
    auto finish = [&] {
        if (threadIdx.x == 0) {
            __threadfence();
            if (atomicAdd(e.L.counters + kCounterEvalDone, 1) == (int)gridDim.x - 1) {
                e.L.counters[kCounterEvalClaim] = 0;
                e.L.counters[kCounterEvalDone] = 0;
            }
        }
    };
    int item = blockIdx.x;
    if (item >= nItems) {
        finish();
        return;
    }
    int next = item + (int)gridDim.x;
    load_twiddles<T, N>(tw, e.k.tw);
    for (int h = threadIdx.x; h < nH; h += THREADS) hpos[h] = (uint16_t)e.hPos[h];
    for (int q = threadIdx.x; q < n2; q += THREADS) amp[q] = e.k.A[q];
    EvalItem it = e.L.eval[item];
    stage_phi<T, N, THREADS>(phiBuf, e.phi + ((size_t)it.p * e.k.I + it.first) * n2);
    cp_async_commit();
    cp_async_wait_all();
    int jj = 0;
    int myClaim = 0;    // thread 0: the item claimed while this one runs
    while (true) {
        const size_t po = (size_t)it.p * e.k.nObj + it.o;
        if (jj == 0) {
            __syncthreads();    // previous item's accumulators written out
            if (threadIdx.x == 0) myClaim = 2 * (int)gridDim.x + atomicAdd(e.L.counters + kCounterEvalClaim, 1);
            for (int h = threadIdx.x; h < nH; h += THREADS) oh[h] = e.Oh[po * nH + h];
#pragma unroll
            for (int i = 0; i < ACC; ++i) acc[i] = Acc4<T>{0, 0, 0, 0};
        }
        // the image after this one (same item, or the first of the block's next item)
        int nextItem = item, nextJj = jj + 1;
        EvalItem nit = it;
        if (nextJj >= it.count) {
            nextItem = next;
            nextJj = 0;
            if (nextItem < nItems) nit = e.L.eval[nextItem];
        }
        const T* phiNext = nextItem < nItems ? e.phi + ((size_t)nit.p * e.k.I + nit.first + nextJj) * n2 : nullptr;
        const int j = it.first + jj;
        const size_t g = (size_t)it.p * e.k.I + j;
        const int ch = e.k.pImgCh[g];
        // a gradient evaluation keeps PF, X and the full OTF for the gradient kernels, unless
        // they recompute them (the OTF is still kept when a buffer for it is given)
        eval_image<T, N, THREADS, ACC, PL>(phiNext, phiBuf, amp, e.k.otfNorm[ch], it.df && !e.k.recompute,
                                  it.df && e.k.S != nullptr, e.k.PF + g * n2, e.k.X + g * N2,
                                  e.k.S + g * N2, e.Dh + g * nH, s, s2, tw, oh, acc, hpos, e.hp.idx, nH);
        if (nextJj == 0) {
            if (threadIdx.x == 0) claimSh = myClaim;
            __syncthreads();
            const int claimed = claimSh;
            Acc4<T>* part = e.part + (size_t)(it.p * e.hp.chunksPerPatch + it.chunk) * nH;
#pragma unroll
            for (int i = 0; i < ACC; ++i) {
                const int h = (int)threadIdx.x + i * THREADS;
                if (h < nH) part[h] = acc[i];
            }
            if (nextItem >= nItems) break;
            item = nextItem;
            it = nit;
            next = claimed;
        }
        jj = nextJj;
    }
    finish();
}

// ----------------------------------------------------------------------------------
// Finite-difference gradient on the half plane (SubImage::gradientFiniteDifference +
// metricChange, subimage.cpp:261-292; the same rearrangement as k_fd):
//     dS = ifft(2 Re(conj(X) dX) + |dX|^2) / N^2,  dX = fft(c PF (exp(i h Z_m) - 1)),
//     dl = -sum [2 Q Re(dS conj G) + |dS|^2 (|D|^2 - Q |O|^2)] / (Q + dq),  G = conj(O)(D - O S).
// dS, G, D, O, S and Q are Hermitian or real and even, so the sum over the support is twice
// the sum over the half plane (the DC term is zero: dS(0) = 0).  One block per image, all
// modes in turn: the per-point factors and c PF are staged in shared memory once per image
// (about 221 KB at N = 88 with 3237 half-plane points);
// X (62 KB per image) is read from L2 for every mode.
// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS, bool RC>
__global__ void __launch_bounds__(THREADS, 1) k_fd_half(EvalParams<T> e) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int n = N / 2, n2 = n * n, N2 = N * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const KParams<T>& kp = e.k;
    const int nH = e.hp.nH;
    // shared memory: two tiles | twiddles | c PF | G (nH) | S (nH) | Q (nH) | |D|^2-Q|O|^2 (nH) |
    //                tile positions (nH)
    cx<T>* a = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* b = a + Tile<N>::ELEMS;
    cx<T>* tw = b + Tile<N>::ELEMS;
    cx<T>* pfs = tw + N;
    cx<T>* hg = pfs + n2;
    cx<T>* hs = hg + nH;
    T* hq = reinterpret_cast<T*>(hs + nH);
    T* hb = hq + nH;
    unsigned short* hpos = reinterpret_cast<unsigned short*>(hb + nH);   // N*(N+1) < 65536
    static_assert(Tile<N>::ELEMS <= 65536, "tile positions are 16-bit");
    __shared__ double red[33];
    const int nWork = *kp.nFdP * kp.I;
    if ((int)blockIdx.x >= nWork) return;
    load_twiddles<T, N>(tw, kp.tw);
    for (int h = threadIdx.x; h < nH; h += THREADS) hpos[h] = (unsigned short)e.hPos[h];
    const T inv = (T)1 / (T)N2;
    for (int w = blockIdx.x; w < nWork; w += gridDim.x) {
        const int p = kp.fdP[w / kp.I], j = w % kp.I;
        const size_t g = (size_t)p * kp.I + j;
        if (j >= kp.pgeo[p].nImg) continue;   // an image slot the patch does not use
        const int o = kp.pImgObj[g];
        const double wgt = kp.objWeight[o];
        const int mc = kp.modeCount[p];
        double* ga = kp.galpha + g * kp.M;
        if (wgt == 0.0) {
            for (int m = threadIdx.x; m < kp.M; m += THREADS) ga[m] = 0.0;
            continue;
        }
        const size_t po = (size_t)p * kp.nObj + o;
        const T c = kp.otfNorm[kp.pImgCh[g]];
        const double hstep = kp.objGradStep[o];
        __syncthreads();    // previous image's staged factors consumed
        const cx<T>* Xg = kp.X + g * N2;
        if constexpr (RC) {
            // recomputed transforms: c PF from the evaluation's phases, X = fft(c PF) into the
            // block's scratch, N^2 S = ifft|X|^2 in tile b (un-centred)
            cx<T>* Xw = kp.Xscr + (size_t)blockIdx.x * N2;
            Xg = Xw;
            for (int i = threadIdx.x; i < Tile<N>::ELEMS; i += THREADS) a[i] = mkc<T>(0, 0);
            __syncthreads();
            for (int q = threadIdx.x; q < n2; q += THREADS) {
                const T amp = kp.A[q];
                cx<T> pf = mkc<T>(0, 0);
                if (amp > (T)0) {
                    T sn, cs;
                    sincos_t<T>(e.phi[g * n2 + q], &sn, &cs);
                    pf = mkc<T>(amp * cs, amp * sn);
                }
                pfs[q] = cscale<T>(pf, c);
                a[(q / n + n / 2) * LDS + q % n + n / 2] = pfs[q];
            }
            __syncthreads();
            fft2d_pp<T, N, -1, THREADS, true>(a, b, tw);
            for (int i = threadIdx.x; i < N2; i += THREADS) {
                const cx<T> X = a[(i / N) * LDS + i % N];
                Xw[i] = X;
                b[(i / N) * LDS + i % N] = mkc<T>(cnorm<T>(X), 0);
            }
            __syncthreads();
            fft2d_pp<T, N, +1, THREADS, false>(b, a, tw);
        } else {
            for (int q = threadIdx.x; q < n2; q += THREADS) pfs[q] = cscale<T>(kp.PF[g * n2 + q], c);
        }
        for (int h = threadIdx.x; h < nH; h += THREADS) {
            const int cidx = e.hp.idx[h];
            const cx<T> S = RC ? cscale<T>(b[hpos[h]], inv) : kp.S[g * N2 + cidx];
            const cx<T> D = kp.D[g * N2 + cidx];
            const cx<T> O = kp.O[po * N2 + cidx];
            const T Q = kp.Qt[po * N2 + cidx];
            hg[h] = cmulc<T>(csub<T>(D, cmul<T>(O, S)), O);
            hs[h] = S;
            // Q < 0 marks the DC point (Q >= gamma > 0 elsewhere)
            hq[h] = (cidx == (N / 2) * N + N / 2) ? (T)-1 : Q;
            hb[h] = cnorm<T>(D) - Q * cnorm<T>(O);
        }
        for (int m = 0; m < kp.M; ++m) {
            if (m >= mc) {
                if (threadIdx.x == 0) ga[m] = 0.0;
                continue;
            }
            const T* Zm = kp.Z + (size_t)m * n2;
            __syncthreads();    // staged factors visible, previous mode's tiles consumed
            // c PF (exp(i t) - 1), t = h Z_m, embedded in tile a for the core
            for (int q = threadIdx.x; q < n2; q += THREADS) {
                const T t = (T)hstep * Zm[q];
                T sh, ch2, sn, cs;
                sincos_t<T>(t * (T)0.5, &sh, &ch2);
                sincos_t<T>(t, &sn, &cs);
                a[(q / n + N / 4) * LDS + q % n + N / 4] = cmul<T>(pfs[q], mkc<T>((T)-2 * sh * sh, sn));
            }
            __syncthreads();
            half_plane_core<T, N, THREADS>(
                a, b, tw,
                [&](int e, int x, cx<T> v) {
                    const cx<T> x0 = Xg[e * N + x];
                    return (T)2 * (x0.x * v.x + x0.y * v.y) + cnorm<T>(v);
                },
                [] {}, [] {}, [] {}, [] {});
            T dl = 0;
            for (int h = threadIdx.x; h < nH; h += THREADS) {
                const T Q = hq[h];
                if (Q < (T)0) continue;
                const cx<T> dS = cscale<T>(a[hpos[h]], inv);
                const cx<T> S = hs[h], G = hg[h];
                const T dS2 = cnorm<T>(dS);
                const T dq = (T)2 * (S.x * dS.x + S.y * dS.y) + dS2;
                const T num = (T)2 * Q * (dS.x * G.x + dS.y * G.y) + dS2 * hb[h];
                dl -= num / (Q + dq);
            }
            const double tot = 2.0 * block_sum<THREADS>((double)dl, red);
            if (threadIdx.x == 0) ga[m] = wgt * (tot / (double)N2 / hstep * wgt);
        }
    }
}

// ----------------------------------------------------------------------------------
// Per-object reduction over the chunks (fixed order) and the object metric: one warp per
// (object, tile of kReduceTile points, four per lane); each lane adds its points' terms and
// the warp adds the lanes' by a fixed shuffle tree, as float-float numbers (about 48 bits, on
// the FP32 pipe: GB300's FP64 pipe is narrow), and the tile's sum is stored in double; the
// solver adds the tiles in order.  mode 1 (gradient) and 2 (refresh) replace O' by the exact
// object O of this point; mode 1 also writes O and Q on the full plane for the gradient
// kernels.
// ----------------------------------------------------------------------------------
template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_reduce(EvalParams<T> e) {
    constexpr int WPB = THREADS / 32;
    constexpr int PER_LANE = kReduceTile / 32;
    static_assert(THREADS % 32 == 0 && kReduceTile % 32 == 0, "tiles are warps");
    const int nItems = *e.L.nPo * e.nTilesH;
    const int nH = e.hp.nH;
    const int lane = threadIdx.x & 31;
    for (int w = blockIdx.x * WPB + threadIdx.x / 32; w < nItems; w += gridDim.x * WPB) {
        const PoItem it = e.L.po[w / e.nTilesH];
        const int tile = w % e.nTilesH;
        const size_t po = (size_t)it.p * e.k.nObj + it.o;
        const T gam = (T)e.k.gamma[po];
        const int c0 = e.hp.objChunk0[po];
        const int nc = (e.k.pObjCount[po] + e.hp.chunkSize - 1) / e.hp.chunkSize;
        const Acc4<T>* base = e.part + (size_t)(it.p * e.hp.chunksPerPatch + c0) * nH;
        float hi = 0.f, lo = 0.f;
#pragma unroll
        for (int k = 0; k < PER_LANE; ++k) {
            const int h = tile * kReduceTile + k * 32 + lane;
            if (h < nH) {
                T R = 0, Q = 0, Pr = 0, Pi = 0;
                for (int c = 0; c < nc; ++c) {
                    const Acc4<T> u = base[(size_t)c * nH + h];
                    R += u.r; Q += u.q; Pr += u.pr; Pi += u.pi;
                }
                const cx<T> oh = e.Oh[po * nH + h];
                const T Qt = gam + Q;
                // conj(P') - gamma O'
                const T dPr = Pr - gam * oh.x, dPi = -Pi - gam * oh.y;
                const T term = R + gam * cnorm<T>(oh) - (dPr * dPr + dPi * dPi) / Qt;
                const int cidx = e.hp.idx[h];
                const bool dc = (cidx == (N / 2) * N + N / 2);
                ff_add(hi, lo, dc ? (float)term : 2.f * (float)term, 0.f);
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
        }
        warp_sum_ff(hi, lo);
        if (lane == 0) e.objMetric[po * e.nTilesH + tile] = (double)hi + (double)lo;
    }
}

}  // namespace rdxg
