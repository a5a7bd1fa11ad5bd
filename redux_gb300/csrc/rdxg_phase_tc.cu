// Mode expansion on the tensor cores: phi = phi_fixed + sum_m alpha_m Z_m
// (SubImage::calcPhi / addToPhi, subimage.cpp:509-544) for every image of the round's work
// list as one GEMM  Phi[pixels x images] = Z'[pixels x K] * B[images x K]^T, where the K
// columns are the fixed phase of each channel followed by the M modes, and B holds a one-hot
// entry for the image's channel followed by its coefficients (so phi_fixed is added by the
// tensor core; K is padded to a multiple of 16 anyway).  The channels come first so that a
// patch using only the first modes of a handle (a ragged batch) has its non-zero products in
// the same K positions as in a handle of its own mode count: the extra modes only add zero
// products at the end.
//
// FP32 operands are split into BF16 parts, x = x0 + x1 (+ x2), each part the BF16 rounding of
// what the previous parts leave, and the products x_i * y_j with i + j < parts are summed by
// tcgen05.mma (kind::f16, FP32 accumulation in tensor memory): two parts give the 3xBF16
// product (relative error ~3 * 2^-18 per term), three parts the 6xBF16 product (~2^-24,
// FP32-like).  The mode tiles are split once per job into the operand layout and copied
// whole into shared memory by the bulk-copy engine; the coefficients are staged with cp.async
// and split by the block into shared memory.  The epilogue reads the accumulators from tensor
// memory (one pixel per thread, 32 images per load) and writes phi coalesced along the pixels.
#include "rdxg_launch.h"
#include "rdxg_tc.cuh"

namespace rdxg {

namespace {

constexpr int kTcRows = 128;     // pixels per tile (MMA M)
constexpr int kTcThreads = 256;  // eight warps: two per quarter of the accumulator lanes

// Zt[tile][part][kmajor(r, k)] for r < 128 pixels of the tile: k < C the channels' fixed
// phases, C <= k < C + M the modes, zero elsewhere.
__global__ void k_tc_pack_modes(const float* __restrict__ Z, const float* __restrict__ phiFixed, int M, int C,
                                int n2, int KP, int parts, int nTiles, __nv_bfloat16* __restrict__ out) {
    const size_t per = (size_t)kTcRows * KP;
    const size_t total = (size_t)nTiles * per;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
        const int tile = (int)(i / per);
        const int e = (int)(i % per);
        const int r = e % kTcRows, k = e / kTcRows;
        const int q = tile * kTcRows + r;
        float rest = 0.f;
        if (q < n2 && k < C) rest = phiFixed[(size_t)k * n2 + q];
        else if (q < n2 && k < C + M) rest = Z[(size_t)(k - C) * n2 + q];
        __nv_bfloat16* dst = out + (size_t)tile * parts * per + tc::kmajor_off(r, k, kTcRows);
        for (int pt = 0; pt < parts; ++pt) {
            const __nv_bfloat16 b = __float2bfloat16_rn(rest);
            dst[(size_t)pt * per] = b;
            rest -= __bfloat162float(b);
        }
    }
}

// Splits 8 consecutive values into BF16 parts and stores each part's 16 bytes (one row of a
// core matrix) at dst + pt * partStride.
__device__ __forceinline__ void split_store8(const float (&x)[8], int parts, __nv_bfloat16* dst, size_t partStride) {
    float rest[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) rest[e] = x[e];
    for (int pt = 0; pt < parts; ++pt) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const __nv_bfloat162 b = __floats2bfloat162_rn(rest[2 * e], rest[2 * e + 1]);
            rest[2 * e] -= __low2float(b);
            rest[2 * e + 1] -= __high2float(b);
            w[e] = *reinterpret_cast<const uint32_t*>(&b);
        }
        *reinterpret_cast<uint4*>(dst + pt * partStride) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

template <int NTMAX>
__global__ void __launch_bounds__(kTcThreads) k_phase_tc(PhaseTcArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ __align__(8) uint64_t bars[2];   // 0: mode tile copied, 1: products complete
    __shared__ uint32_t tmemBase;
    __shared__ int issued;

    const int KP = a.KP, NT = a.NT, n2 = a.n2, I = a.I, M = a.M, C = a.nCh, G = a.G, parts = a.parts;
    const int nTiles = (n2 + kTcRows - 1) / kTcRows;
    const int nP = *a.nEvalP;
    const int nWork = ((nP + G - 1) / G) * nTiles;
    if ((int)blockIdx.x >= nWork) return;   // uniform per block, before any barrier

    const uint32_t aBytes = (uint32_t)parts * kTcRows * KP * 2;   // one tile, all parts
    const int bPart = NT * KP;                                     // elements per part of B
    const int IM = I * M;
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    __nv_bfloat16* sB = reinterpret_cast<__nv_bfloat16*>(smem_raw + aBytes);
    float** colPtr = reinterpret_cast<float**>(smem_raw + aBytes + (size_t)parts * bPart * 2);   // [NTMAX]
    int* colCh = reinterpret_cast<int*>(colPtr + NTMAX);                                      // [NTMAX]
    float* sAl = reinterpret_cast<float*>(colCh + NTMAX);                                     // [G][I*M]

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        tc::mbar_init(&bars[0], 1);
        tc::mbar_init(&bars[1], 1);
        tc::mbar_init_fence();
    }
    if (warp == 0) {
        tc::tmem_alloc(&tmemBase, NTMAX);
        tc::tmem_relinquish();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmemBase;
    const uint32_t idesc = tc::idesc_bf16(kTcRows, NT);
    const uint32_t aBase = tc::smem_u32(sA), bBase = tc::smem_u32(sB);
    const int kChunks = KP / 8;

    int tileLoaded = -1;
    uint32_t phA = 0, phM = 0;
    bool copyPending = false, mmaPending = false, ok = true;
    for (int w = blockIdx.x; w < nWork; w += gridDim.x) {
        const int tile = w % nTiles, grp = w / nTiles;
        const int q0 = tile * kTcRows;
        if (tile != tileLoaded) {
            // the previous products have completed (waited for below): the tile may be replaced
            if (tid == 0) {
                tc::mbar_arrive_expect_tx(&bars[0], aBytes);
                tc::bulk_g2s(sA, a.Zt + (size_t)tile * parts * kTcRows * KP, aBytes, &bars[0]);
            }
            copyPending = true;
            tileLoaded = tile;
        }
        // the group's coefficients (I*M contiguous values per patch), all copies in flight at once
        const int nSlots = min(G, nP - grp * G);
        for (int s = 0; s < nSlots; ++s) {
            const float* src = a.alphaEff + (size_t)a.evalP[grp * G + s] * IM;
            for (int i = tid; i < IM; i += kTcThreads) cp_async4(sAl + s * IM + i, src + i);
        }
        cp_async_commit();
        // the group's images: column c = slot * I + j, slot = patch of the group
        for (int c = tid; c < NTMAX; c += kTcThreads) {
            const int s = c / I, j = c - s * I;
            const bool valid = s < nSlots;
            colPtr[c] = valid ? a.phi + ((size_t)a.evalP[grp * G + s] * I + j) * n2 : nullptr;
            colCh[c] = valid ? a.imgCh[(size_t)a.evalP[grp * G + s] * I + j] : -1;
        }
        cp_async_wait_all();
        __syncthreads();
        // B operand: coefficients and the channel's one-hot entry, split into parts, zero
        // beyond the valid images; each thread one core-matrix row (8 values of K) per part
        for (int u = tid; u < NT * kChunks; u += kTcThreads) {
            const int c = u / kChunks, k0 = (u - c * kChunks) * 8;
            const int s = c / I;
            const float* src = sAl + s * IM + (c - s * I) * M;
            const bool valid = s < nSlots;
            const int kOne = valid ? colCh[c] : -1;
            float x[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
                const int k = k0 + e;
                x[e] = (valid && k >= C && k < C + M) ? src[k - C] : (k == kOne ? 1.f : 0.f);
            }
            split_store8(x, parts, sB + tc::kmajor_off(c, k0, NT), (size_t)bPart);
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        if (tid == 0) {
            issued = 0;
            const bool have = !copyPending || tc::mbar_wait(&bars[0], phA);
            if (have) {
                tc::fence_after_sync();
                // every product of the smaller parts first, over all of K, so that they are
                // summed while the accumulator is still small; the leading products last
                uint32_t acc = 0;
                for (int sum = parts - 1; sum >= 0; --sum) {
                    for (int i = 0; i <= sum; ++i) {
                        const int j = sum - i;
                        for (int kb = 0; kb < KP / 16; ++kb) {
                            const uint64_t ad = tc::smem_desc(
                                aBase + (uint32_t)(i * kTcRows * KP * 2 + kb * kTcRows * 32), tc::kLbo, tc::kSbo);
                            const uint64_t bd =
                                tc::smem_desc(bBase + (uint32_t)(j * bPart * 2 + kb * NT * 32), tc::kLbo, tc::kSbo);
                            tc::mma_bf16(tmem, ad, bd, idesc, acc);
                            acc = 1;
                        }
                    }
                }
                tc::mma_commit(&bars[1]);
                issued = 1;
            } else {
                atomicExch(a.status, 1);
            }
        }
        __syncthreads();
        if (copyPending && issued) { phA ^= 1; copyPending = false; }
        if (!issued) { ok = false; break; }
        mmaPending = true;
        const bool done = tc::mbar_wait(&bars[1], phM);
        if (!__syncthreads_and(done)) {
            if (tid == 0) atomicExch(a.status, 2);
            ok = false;
            break;
        }
        phM ^= 1;
        mmaPending = false;
        tc::fence_after_sync();
        // warp w reads lanes 32 (w % 4) .. + 31 (its pixels) and every other chunk of 32 images
        const int quarter = warp & 3;
        const int q = q0 + quarter * 32 + lane;
        for (int c0 = (warp >> 2) * 32; c0 < NT; c0 += 64) {
            float v[32];
            tc::tmem_ld32(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)c0, v);
            if (q < n2) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    float* dst = colPtr[c0 + j];
                    if (dst) dst[q] = v[j];
                }
            }
        }
        tc::fence_before_sync();
        __syncthreads();   // accumulators and column tables consumed before the next item
    }
    if (!ok) {
        // let whatever is still in flight land before the memory goes away (bounded again)
        if (tid == 0) {
            if (copyPending) tc::mbar_wait(&bars[0], phA);
            if (mmaPending) tc::mbar_wait(&bars[1], phM);
        }
    }
    __syncthreads();
    tc::fence_after_sync();
    if (warp == 0) tc::tmem_dealloc(tmem, NTMAX);
}

template <int NTMAX>
size_t phase_tc_smem(int KP, int NT, int parts, int G, int I, int M) {
    return (size_t)parts * kTcRows * KP * 2 + (size_t)parts * NT * KP * 2 + (size_t)NTMAX * 12 +
           (size_t)G * I * M * 4;
}

}  // namespace

PhaseTcPlan phase_tc_plan(int I, int M, int n2, int nCh, int parts, int numSMs) {
    PhaseTcPlan p{};
    if (I < 1 || I > 256 || M < 1 || M > 256 || parts < 2 || parts > 3) return p;
    p.ntmax = I <= 128 ? 128 : 256;
    p.G = p.ntmax / I;
    p.NT = (p.G * I + 15) / 16 * 16;
    p.KP = (M + nCh + 15) / 16 * 16;   // modes, then one fixed-phase column per channel
    p.parts = parts;
    p.nTiles = (n2 + kTcRows - 1) / kTcRows;
    p.smem = p.ntmax == 128 ? phase_tc_smem<128>(p.KP, p.NT, parts, p.G, I, M)
                            : phase_tc_smem<256>(p.KP, p.NT, parts, p.G, I, M);
    if (p.smem > kMaxSmem) return PhaseTcPlan{};
    int occ = 0;
    cudaError_t e;
    // all of the unified L1 as shared memory, so that several blocks fit per SM
    auto setup = [&](auto kern) {
        cudaError_t r = raise_smem_limit(kern, p.smem);
        if (r == cudaSuccess)
            r = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     (int)cudaSharedmemCarveoutMaxShared);
        if (r == cudaSuccess) r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kTcThreads, p.smem);
        return r;
    };
    e = p.ntmax == 128 ? setup(k_phase_tc<128>) : setup(k_phase_tc<256>);
    if (e != cudaSuccess || occ < 1) return PhaseTcPlan{};
    p.occ = occ;
    // The query answers 1 for this kernel although shared memory, registers and threads allow
    // more; size the grid by the shared memory (228 KB per SM, 1 KB reserved per block) and by
    // the 512 tensor-memory columns of an SM.  Blocks beyond what fits simply queue.
    const int bySmem = (228 * 1024) / (int)(p.smem + 1024 + 256);
    const int byTmem = 512 / p.ntmax;
    occ = bySmem < byTmem ? bySmem : byTmem;
    if (occ < 1) occ = 1;
    // a multiple of the pixel tiles, so that each block keeps one mode tile
    int grid = numSMs * occ;
    grid = grid / p.nTiles * p.nTiles;
    if (grid < p.nTiles) grid = p.nTiles;
    p.grid = grid;
    p.zElems = (size_t)p.nTiles * parts * kTcRows * p.KP;
    p.valid = 1;
    return p;
}

void launch_tc_pack_modes(const float* Z, const float* phiFixed, int M, int C, int n2, const PhaseTcPlan& p,
                          __nv_bfloat16* out, cudaStream_t st) {
    k_tc_pack_modes<<<256, 256, 0, st>>>(Z, phiFixed, M, C, n2, p.KP, p.parts, p.nTiles, out);
}

void launch_phase_tc(const PhaseTcArgs& a, const PhaseTcPlan& p, cudaStream_t st) {
    if (p.ntmax == 128) k_phase_tc<128><<<p.grid, kTcThreads, p.smem, st>>>(a);
    else k_phase_tc<256><<<p.grid, kTcThreads, p.smem, st>>>(a);
}

}  // namespace rdxg
