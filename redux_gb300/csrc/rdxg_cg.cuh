// Device side of the per-patch optimiser: one thread block per patch; its first warp runs the
// state machine of cg_machine.h (scalar logic replicated in the warp's lanes, vector
// operations warp-parallel, all sums in double in a fixed order), the block maps the point of the next
// evaluation through the null-space map (Constraints::reverseAndAdd,
// constraints.hpp:141-146) and the gradient back (Constraints::apply, 128-133), and
// performs the integer image re-shifts between mode stages (SubImage::adjustShifts,
// subimage.cpp:444-480).
#pragma once

#include "cg_machine.h"
#include "rdxg_eval.cuh"
#include "rdxg_kernels.cuh"

namespace rdxg {

// Vector operations of the state machine, run by one warp (warp 0 of the block): the scalar
// logic (FP64, including divisions) is then issued by one warp instead of every warp of the
// block, on GB300's narrow FP64 pipe.  Sums: a fixed shuffle tree into lane 0, broadcast, so
// every lane holds the same bits.
struct WarpVec {
    int n;
    // with the vectors staged in shared memory: their base and stride, and a bit per vector
    // written (in every lane), so that only those are copied back
    double* base = nullptr;
    int stride = 0;
    unsigned dirty = 0;
    __device__ void mark(const double* d) {
        if (base) dirty |= 1u << (int)((d - base) / stride);
    }
    __device__ static double wsum(double a) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
        return __shfl_sync(0xffffffffu, a, 0);
    }
    __device__ static int lane() { return threadIdx.x & 31; }
    __device__ void copy(double* d, const double* s) {
        for (int i = lane(); i < n; i += 32) d[i] = s[i];
        mark(d);
        __syncwarp();
    }
    __device__ void zero(double* d) {
        for (int i = lane(); i < n; i += 32) d[i] = 0.0;
        mark(d);
        __syncwarp();
    }
    __device__ double nrm2(const double* v) {
        double a = 0;
        for (int i = lane(); i < n; i += 32) a += v[i] * v[i];
        return sqrt(wsum(a));
    }
    __device__ double dot(const double* x, const double* y) {
        double a = 0;
        for (int i = lane(); i < n; i += 32) a += x[i] * y[i];
        return wsum(a);
    }
    __device__ double pr_update(double* g0, const double* g) {
        double a = 0;
        for (int i = lane(); i < n; i += 32) {
            const double t = g0[i] - g[i];
            a += t * g[i];
            g0[i] = t;
        }
        mark(g0);
        __syncwarp();
        return wsum(a);
    }
    __device__ void dir_update(double* p, const double* g, double beta) {
        for (int i = lane(); i < n; i += 32) p[i] = g[i] - beta * p[i];
        mark(p);
        __syncwarp();
    }
    __device__ void step(double* x1, const double* x, const double* p, double s) {
        for (int i = lane(); i < n; i += 32) x1[i] = x[i] + s * p[i];
        mark(x1);
        __syncwarp();
    }
};

template <typename T>
struct CgArgs {
    CgParams prm;
    int32_t P, I, M, nObj, nPar, nTiles, ps;
    CgState* states;        // [P]
    double* vec;            // [P][5][nFree]: x, p, g, g0, x1
    double* metrics;        // [P][max_metrics]
    double* alpha;          // [P][nPar]
    double* alphaOff;       // [P][nPar]
    float* alphaOffF;       // [P][nPar] alphaOff rounded to float (the FP32 map's offsets)
    const double* galpha;   // [P][nPar]
    const double* partial;  // [P][nObj][nTiles]
    const double* objWeight;
    // null-space maps, by parameter row and by free column: every patch shape's, one after the
    // other (PatchGeo::rowBase, colBase); rows in the handle's layout (image slot * M + mode)
    const PatchGeo* pgeo;   // [P]
    const int32_t* rowPtr; const int32_t* rowCol; const double* rowVal;
    const float* rowVal32;  // FP32 copy of rowVal
    int32_t x1Smem;         // FP32 metric-request map enabled (dynamic shared memory n_free floats)
    // staged form (CgStageLayout): the patch's vectors, object metric tiles and weights and
    // object tables copied into shared memory when the kernel starts; stageMap: the entries of
    // its row map as well (FP32 map, at most kCgRowsPerThread rows per thread)
    int32_t stage, stageMap, maxNnz;
    const int32_t* colPtr; const int32_t* colRow; const double* colVal;
    const double* curTilt;  // [P][I][2] (y, x): currentTiltOffset of each image
    const double* resAlpha; // [P][I][2] (y, x): channel residual tilt (phi_channel term)
    int32_t tiltX, tiltY;
    T* alphaEff;            // [P][I][M]
    int32_t* req;
    int32_t* gmethod;
    int32_t* modeCount;
    int32_t* active;
    // fused evaluation path (FP32): object metrics, work lists, reference-object state
    int32_t fused;
    const double* objMetric;       // [P][nObj][nTilesH] per-tile partial sums
    int32_t nTilesH;
    Lists L;
    int32_t chunkSize, chunksPerPatch;
    const int32_t* objChunk0;      // [P][nObj]
    const int32_t* objFirst;       // [P][nObj]
    const int32_t* objCount;       // [P][nObj]
    int32_t* aux;                  // [P][2]: reference object valid, refresh pending
    const double* regW;            // [nPar] REG_ALPHA weights, or null
    int32_t phaseList;             // general path: list the evaluated patches (tensor-core expansion)
};

// alpha = offset + N x1; alpha_eff = alpha + currentTiltOffset - residual for the tilt modes
// (the residual is what Channel::initPatch adds to phi_channel, channel.cpp:916-939)
template <typename T, int THREADS>
__device__ void map_point(const CgArgs<T>& a, int p, const double* x1, bool writeEff = true) {
    const double* off = a.alphaOff + (size_t)p * a.nPar;
    double* al = a.alpha + (size_t)p * a.nPar;
    T* ae = a.alphaEff + (size_t)p * a.nPar;
    const int32_t* rp = a.rowPtr + a.pgeo[p].rowBase;
    for (int r = threadIdx.x; r < a.nPar; r += THREADS) {
        double v = off[r];
        for (int e = rp[r]; e < rp[r + 1]; ++e) v += a.rowVal[e] * x1[a.rowCol[e]];
        al[r] = v;
        if (!writeEff) continue;
        const int j = r / a.M, m = r % a.M;
        double ve = v;
        const size_t b = ((size_t)p * a.I + j) * 2;
        if (m == a.tiltX) ve += a.curTilt[b + 1] - a.resAlpha[b + 1];
        else if (m == a.tiltY) ve += a.curTilt[b + 0] - a.resAlpha[b + 0];
        ae[r] = (T)ve;
    }
    __syncthreads();
}

// The FP32 path's metric and gradient requests: alphaEff in FP32 arithmetic (it is rounded to
// FP32 for the evaluation anyway), with the point staged in shared memory as float and the
// offsets kept as float.  GB300 issues an FP64 instruction in 64 cycles per warp and a
// double-to-float conversion in about 80, whatever the number of active lanes, which makes
// the FP64 map the largest cost of the solver kernel; the FP64 alpha is formed by map_point
// (without alphaEff) for every gradient, re-shift and final point, where it is used.
template <typename T, int THREADS>
__device__ void map_point_f32(const CgArgs<T>& a, int p, const double* x1, float* xs) {
    const int nF = a.pgeo[p].nFree;
    if (xs) {
        for (int c = threadIdx.x; c < nF; c += THREADS) xs[c] = (float)x1[c];
        __syncthreads();
    }
    const float* off = a.alphaOffF + (size_t)p * a.nPar;
    T* ae = a.alphaEff + (size_t)p * a.nPar;
    const int32_t* rp = a.rowPtr + a.pgeo[p].rowBase;
    for (int r = threadIdx.x; r < a.nPar; r += THREADS) {
        float v = 0.f;
        for (int e = rp[r]; e < rp[r + 1]; ++e)
            v = fmaf(a.rowVal32[e], xs ? xs[a.rowCol[e]] : (float)x1[a.rowCol[e]], v);
        v += off[r];
        const int j = r / a.M, m = r % a.M;
        const size_t b = ((size_t)p * a.I + j) * 2;
        if (m == a.tiltX) v += (float)(a.curTilt[b + 1] - a.resAlpha[b + 1]);
        else if (m == a.tiltY) v += (float)(a.curTilt[b + 0] - a.resAlpha[b + 0]);
        ae[r] = (T)v;
    }
    __syncthreads();
}

// Arguments of the re-shifts (SubImage::adjustShifts of patches that request one).
struct ShiftArgs {
    int32_t P, I, M, nObj, ps, cs, margin, tiltX, tiltY;
    const int32_t* req;
    const double* alpha;     // [P][I*M]
    double* tiltOff;         // [P][I][2] currentTiltOffset (y, x)
    int32_t* shift;          // [P][I][2]
    uint8_t* reinit;         // [P][I]
    const int32_t* imgObj;   // [P][I]
    const PatchGeo* pgeo;     // [P]
    int32_t* aux;            // [P][2] reference object valid flag (cleared on re-initialisation)
    double J[2][2], Jinv[2][2];
    // rounds run as a CUDA graph: the conditions of the graph's optional kernels (image
    // re-initialisation, adjoint, finite differences), set once per round from the work-list
    // counters, and the kernel launches of the round added to launchCount
    int32_t useConditions;
    cudaGraphConditionalHandle condPrep, condAdjoint, condFd;
    const int32_t* counters;
    int32_t fixedLaunches;
    int32_t prepLaunches;       // kernels of the re-initialisation node (plane fit + preparation)
    unsigned long long* launchCount;
};

// adjustShifts of one patch's images (SubImage::adjustShifts, subimage.cpp:444-480) when its
// request is a re-shift; marks the images of every object that has a shifted image for
// re-initialisation (Object::reInitialize), and clears the marks otherwise.  All threads of
// the block.
__device__ __forceinline__ void shift_patch(const ShiftArgs& a, int p, int req) {
    if (req != REQ_SHIFT) {
        for (int j = threadIdx.x; j < a.I; j += blockDim.x) a.reinit[(size_t)p * a.I + j] = 0;
        return;
    }
    const int nImg = a.pgeo[p].nImg;
    __shared__ int objShifted[64];
    for (int o = threadIdx.x; o < a.nObj; o += blockDim.x) objShifted[o] = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nImg; j += blockDim.x) {
        const size_t gi = (size_t)p * a.I + j;
        const double* al = a.alpha + gi * a.M;
        if (a.tiltX < 0 || a.tiltY < 0) continue;
        const double ay = al[a.tiltY] + a.tiltOff[gi * 2 + 0];
        const double ax = al[a.tiltX] + a.tiltOff[gi * 2 + 1];
        const double sy = ax * a.J[1][0] + ay * a.J[1][1];
        const double sx = ax * a.J[0][0] + ay * a.J[0][1];
        const int want[2] = {-(int)llround(sy), -(int)llround(sx)};
        int act[2] = {0, 0};
        for (int d = 0; d < 2; ++d) {
            int nsh = want[d];
            if (!nsh) continue;
            const int first = a.margin + a.shift[gi * 2 + d];
            const int last = first + a.ps - 1;
            if (nsh + first < 0) nsh = -first;
            if (abs(nsh + last) >= a.cs) nsh = a.cs - last - 1;
            act[d] = nsh;
        }
        if (act[0] || act[1]) {
            a.shift[gi * 2 + 0] += act[0];
            a.shift[gi * 2 + 1] += act[1];
            a.tiltOff[gi * 2 + 0] += act[1] * a.Jinv[1][0] + act[0] * a.Jinv[1][1];
            a.tiltOff[gi * 2 + 1] += act[1] * a.Jinv[0][0] + act[0] * a.Jinv[0][1];
            atomicExch(&objShifted[a.imgObj[gi]], 1);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < a.I; j += blockDim.x) {
        const int sh = j < nImg ? objShifted[a.imgObj[(size_t)p * a.I + j]] : 0;
        a.reinit[(size_t)p * a.I + j] = sh ? 1 : 0;
        if (sh && a.aux) a.aux[2 * p + 0] = 0;
    }
}

// The conditions of the round's optional graph nodes (image re-initialisation, adjoint,
// finite differences) from its work-list counters, and the kernel launches of the round
// added to launchCount.  One thread, once every solver-kernel block of the round is done.
__device__ __forceinline__ void set_round_conditions(const ShiftArgs& a) {
    const unsigned prep = atomicAdd(const_cast<int32_t*>(a.counters) + kCounterShift, 0) > 0,
                   adj = atomicAdd(const_cast<int32_t*>(a.counters) + kCounterGrad, 0) > 0,
                   fd = atomicAdd(const_cast<int32_t*>(a.counters) + kCounterFd, 0) > 0;
    cudaGraphSetConditional(a.condPrep, prep);
    cudaGraphSetConditional(a.condAdjoint, adj);
    cudaGraphSetConditional(a.condFd, fd);
    *a.launchCount += (unsigned long long)(a.fixedLaunches + prep * a.prepLaunches + adj + fd);
}

// Shared-memory layout (bytes) of the staged solver kernel: the patch's five vectors, its
// object metric tiles, the object weights, its reference-object flags and object tables, and
// (stageMap) its row map (row pointers, entry values and columns), alpha offsets (float), the
// tilt terms of its images (currentTiltOffset, channel residual) and the point as float.
struct CgStageLayout {
    size_t om, ow, off, tilt, ints, rp, ec, ev, xs, total;
    __host__ __device__ CgStageLayout(int stride, int nObj, int nT, int stageMap, int nPar, int I, int maxNnz) {
        const size_t d = sizeof(double), i4 = sizeof(int32_t);
        om = (size_t)5 * stride * d;
        ow = om + (size_t)nObj * nT * d;
        off = ow + (size_t)nObj * d;
        tilt = (off + (stageMap ? (size_t)nPar * sizeof(float) : 0) + 7) & ~(size_t)7;
        ints = tilt + (stageMap ? (size_t)4 * I * d : 0);
        rp = ints + (size_t)(2 + 3 * nObj) * i4;
        ec = rp + (stageMap ? (size_t)(nPar + 1) * i4 : 0);
        ev = ec + (stageMap ? (size_t)maxNnz * i4 : 0);
        xs = ev + (stageMap ? (size_t)maxNnz * sizeof(float) : 0);
        total = xs + (stageMap ? (size_t)stride * sizeof(float) : 0);
    }
};

// The FP32 map of the staged kernel: the same arithmetic as map_point_f32, every operand in
// shared memory (rps: the patch's row pointers, ec/ev: its entries from entry e0 on, offs: its
// alpha offsets, tilt: [2][I][2] current tilt offsets and channel residuals, xs: room for the
// point as float, converted once per free parameter).
template <typename T, int THREADS>
__device__ void map_rows_staged(const CgArgs<T>& a, int p, const double* x1, const int32_t* rps, const int32_t* ec,
                                const float* ev, const float* offs, const double* tilt, float* xs, int nF) {
    for (int c = threadIdx.x; c < nF; c += THREADS) xs[c] = (float)x1[c];
    __syncthreads();
    T* ae = a.alphaEff + (size_t)p * a.nPar;
    const int e0 = rps[0];
    const double* cur = tilt;
    const double* res = tilt + 2 * a.I;
    for (int r = threadIdx.x; r < a.nPar; r += THREADS) {
        float v = 0.f;
        for (int e = rps[r] - e0; e < rps[r + 1] - e0; ++e) v = fmaf(ev[e], xs[ec[e]], v);
        v += offs[r];
        const int j = r / a.M, m = r % a.M;
        if (m == a.tiltX) v += (float)(cur[2 * j + 1] - res[2 * j + 1]);
        else if (m == a.tiltY) v += (float)(cur[2 * j + 0] - res[2 * j + 0]);
        ae[r] = (T)v;
    }
    __syncthreads();
}

// append the chunks and objects of patch p to the evaluation work lists; cnt, first, ch0: the
// patch's object image counts, first images and first chunks
template <typename T>
__device__ void enqueue_eval(const CgArgs<T>& a, int p, int rq, int mode, const int32_t* cnt, const int32_t* first,
                             const int32_t* ch0, int chunks) {
    // one reservation per list (the atomics go out together), then the writes
    const int kp = atomicAdd(a.L.nEvalP, 1);
    const int k0 = atomicAdd(a.L.nEval, chunks);
    const int j0 = atomicAdd(a.L.nPo, a.nObj);
    a.L.evalP[kp] = p;
    for (int o = 0; o < a.nObj; ++o) {
        const int nc = (cnt[o] + a.chunkSize - 1) / a.chunkSize;
        for (int c = 0; c < nc; ++c) {
            EvalItem it;
            it.p = p; it.o = o;
            it.first = first[o] + c * a.chunkSize;
            it.count = min(a.chunkSize, cnt[o] - c * a.chunkSize);
            it.chunk = ch0[o] + c;
            it.df = (rq == REQ_DF) ? 1 : 0;
            a.L.eval[k0 + ch0[o] + c] = it;
        }
        PoItem pi;
        pi.p = p; pi.o = o; pi.mode = mode;
        a.L.po[j0 + o] = pi;
    }
}

// One block per patch.  ST (staged): the patch's vectors, object metric tiles, object
// weights and tables (and, with stageMap, its row map) are copied into shared memory with
// cp.async as the kernel starts, so that the state machine's vector operations, the object
// sums, the map and the work-list appends wait on shared memory instead of chains of
// dependent global loads; the vectors the round wrote are copied back at the end.  The
// arithmetic and its order are the same in both forms.
// At the end every block re-shifts its own patch when that is its request (shift_patch) and,
// in a solve graph, the last block of the round sets the conditions of the round's optional
// nodes from the work-list counters (set_round_conditions).
template <typename T, int THREADS, bool ST>
__global__ void __launch_bounds__(THREADS) k_cg(CgArgs<T> a, ShiftArgs sa) {
    const int p = blockIdx.x;
    auto finish = [&](int req) {
        shift_patch(sa, p, req);
        if (sa.useConditions) {
            __syncthreads();    // the block's appends to the work lists are done
            if (threadIdx.x == 0) {
                __threadfence();
                if (atomicAdd(a.L.counters + kCounterCgDone, 1) == (int)gridDim.x - 1) {
                    __threadfence();
                    set_round_conditions(sa);
                }
            }
        }
    };
    __shared__ double fsh;
    __shared__ double objSum[64];
    __shared__ int32_t pcShared, reqShared;
    __shared__ unsigned dirtyShared;
    extern __shared__ __align__(16) unsigned char cg_smem[];
    // the state is read by the first warp, which runs the machine; the block needs pc and req
    CgState st;
    if (threadIdx.x < 32) st = a.states[p];
    const PatchGeo pg = a.pgeo[p];
    const int nF = pg.nFree;
    const int32_t* rp = a.rowPtr + pg.rowBase;
    const int32_t* cp = a.colPtr + pg.colBase;
    // the patch's vectors, nF long, at the stride of the handle's largest (prm.n_free)
    const int stride = a.prm.n_free;
    double* const vg = a.vec + (size_t)p * 5 * stride;
    const int nT = a.fused ? a.nTilesH : a.nTiles;
    const double* om = (a.fused ? a.objMetric : a.partial) + (size_t)p * a.nObj * nT;
    const double* ow = a.objWeight;
    const int32_t* tabs = nullptr;      // staged: aux flags, object counts, first images, first chunks
    double* vb = vg;                    // where the machine works on the vectors
    const CgStageLayout lay(stride, a.nObj, nT, a.stageMap, a.nPar, a.I, a.maxNnz);
    int32_t* rps = reinterpret_cast<int32_t*>(cg_smem + lay.rp);
    int32_t* ec = reinterpret_cast<int32_t*>(cg_smem + lay.ec);
    float* ev = reinterpret_cast<float*>(cg_smem + lay.ev);
    float* offs = reinterpret_cast<float*>(cg_smem + lay.off);
    double* tilt = reinterpret_cast<double*>(cg_smem + lay.tilt);
    int e0 = 0;
    if (ST) {
        double* vs = reinterpret_cast<double*>(cg_smem);
        for (int i = threadIdx.x; i < 5 * nF; i += THREADS) {
            const int k = i / nF, c = i - k * nF;
            cp_async8(vs + (size_t)k * stride + c, vg + (size_t)k * stride + c);
        }
        double* oms = reinterpret_cast<double*>(cg_smem + lay.om);
        double* ows = reinterpret_cast<double*>(cg_smem + lay.ow);
        int32_t* ints = reinterpret_cast<int32_t*>(cg_smem + lay.ints);
        for (int i = threadIdx.x; i < a.nObj * nT; i += THREADS) cp_async8(oms + i, om + i);
        for (int i = threadIdx.x; i < a.nObj; i += THREADS) cp_async8(ows + i, a.objWeight + i);
        if (a.fused) {
            if (threadIdx.x < 2) cp_async4(ints + threadIdx.x, a.aux + 2 * p + threadIdx.x);
            for (int i = threadIdx.x; i < a.nObj; i += THREADS) {
                const size_t po = (size_t)p * a.nObj + i;
                cp_async4(ints + 2 + i, a.objCount + po);
                cp_async4(ints + 2 + a.nObj + i, a.objFirst + po);
                cp_async4(ints + 2 + 2 * a.nObj + i, a.objChunk0 + po);
            }
        }
        cp_async_commit();
        vb = vs; om = oms; ow = ows; tabs = ints;
        if (a.stageMap) {
            // the FP32 map's operands: row pointers, alpha offsets, tilt terms (the entries
            // follow once their range is known)
            for (int r = threadIdx.x; r <= a.nPar; r += THREADS) cp_async4(rps + r, rp + r);
            const float* off = a.alphaOffF + (size_t)p * a.nPar;
            for (int r = threadIdx.x; r < a.nPar; r += THREADS) cp_async4(offs + r, off + r);
            const size_t b = (size_t)p * a.I * 2;
            for (int i = threadIdx.x; i < 2 * a.I; i += THREADS) {
                cp_async8(tilt + i, a.curTilt + b + i);
                cp_async8(tilt + 2 * a.I + i, a.resAlpha + b + i);
            }
            cp_async_commit();
            e0 = rp[0];
        }
    }
    if (threadIdx.x == 0) { pcShared = st.pc; reqShared = st.req; dirtyShared = 0; }
    __syncthreads();
    const int pc0 = pcShared, req0 = reqShared;
    if (ST && a.stageMap) {
        const int e1 = rp[a.nPar];
        for (int e = e0 + (int)threadIdx.x; e < e1; e += THREADS) {
            cp_async4(ev + (e - e0), a.rowVal32 + e);
            cp_async4(ec + (e - e0), a.rowCol + e);
        }
        cp_async_commit();
    }
    double* x = vb;
    double* pv = x + stride;
    double* g = pv + stride;
    double* g0 = g + stride;
    double* x1 = g0 + stride;
    if (pc0 == PC_DONE) {
        if (ST) cp_async_wait_all();
        if (threadIdx.x == 0) a.req[p] = REQ_DONE;
        finish(REQ_DONE);
        return;
    }
    double f = 0;
    if (a.fused && req0 == REQ_F && a.aux[2 * p + 1]) {
        // the last evaluation only refreshed the reference object: repeat the request
        if (ST) cp_async_wait_all();
        if (threadIdx.x == 0) {
            a.aux[2 * p + 0] = 1;
            a.aux[2 * p + 1] = 0;
            a.req[p] = REQ_F;
            atomicAdd(a.active, 1);
            const size_t po = (size_t)p * a.nObj;
            enqueue_eval(a, p, REQ_F, 0, a.objCount + po, a.objFirst + po, a.objChunk0 + po, pg.chunks);
        }
        finish(REQ_F);
        return;
    }
    if (ST) {
        // the vectors, tiles and tables (the row map's entries may still be in flight)
        if (a.stageMap) cp_async_wait_one();
        else cp_async_wait_all();
        __syncthreads();
    }
    if (req0 == REQ_F) {
        // object sums: one warp per object, each lane adds its tiles in order, then a fixed
        // shuffle tree; the objects are added in order
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int o = wid; o < a.nObj; o += THREADS / 32) {
            double m = 0;
            for (int t = lane; t < nT; t += 32) m += om[(size_t)o * nT + t];
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) m += __shfl_down_sync(0xffffffffu, m, off);
            // each object's weighted term in its own warp (the divisions run side by side)
            if (lane == 0) {
                const double w = ow[o];
                objSum[o] = (w != 0.0) ? w * (m / ((double)a.ps * a.ps)) : 0.0;
            }
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum = 0;
            for (int o = 0; o < a.nObj; ++o)
                if (ow[o] != 0.0) sum += objSum[o];
            fsh = sum;
        }
        __syncthreads();
        f = fsh;
        if (a.regW) {
            // REG_ALPHA: + 0.5 sum alpha^2 w at the evaluated point (solver.cpp:804-811), alpha
            // = alpha_offset + N x1 in FP64
            __shared__ double red[33];
            const double* off = a.alphaOff + (size_t)p * a.nPar;
            double part = 0;
            for (int r = threadIdx.x; r < a.nPar; r += THREADS) {
                double v = off[r];
                for (int e = rp[r]; e < rp[r + 1]; ++e) v += a.rowVal[e] * x1[a.rowCol[e]];
                part += 0.5 * v * v * a.regW[r];
            }
            f += block_sum<THREADS>(part, red);
        }
    } else if (req0 == REQ_DF) {
        const double* ga = a.galpha + (size_t)p * a.nPar;
        // REG_ALPHA: the modes not enabled keep alpha * w (the enabled ones are assigned the
        // data term, solver.cpp:860-885)
        const double* al = a.alpha + (size_t)p * a.nPar;
        const int mcount = a.modeCount[p];
        for (int c = threadIdx.x; c < nF; c += THREADS) {
            double v = 0;
            for (int e = cp[c]; e < cp[c + 1]; ++e) {
                const int row = a.colRow[e];
                const double gr = (a.regW && row % a.M >= mcount) ? al[row] * a.regW[row] : ga[row];
                v += a.colVal[e] * gr;
            }
            g[c] = v;
        }
        if (ST && threadIdx.x == 0) dirtyShared |= 1u << 2;
        __syncthreads();
    } else if (req0 == REQ_SHIFT) {
        double* off = a.alphaOff + (size_t)p * a.nPar;
        float* offF = a.alphaOffF + (size_t)p * a.nPar;
        const double* al = a.alpha + (size_t)p * a.nPar;
        for (int r = threadIdx.x; r < a.nPar; r += THREADS) {
            const double v = al[r];
            off[r] = v;
            offF[r] = (float)v;
            if (ST && a.stageMap) offs[r] = (float)v;
        }
        __syncthreads();
    }
    __shared__ int rqShared;
    if (threadIdx.x < 32) {
        WarpVec V{nF};
        if (ST) { V.base = vb; V.stride = stride; }
        CgParams prm = a.prm;       // the patch's own sizes
        prm.n_free = nF;
        prm.n_modes = pg.nMode;
        Machine<WarpVec> mc(prm, st, V, x, pv, g, g0, x1, a.metrics + (size_t)p * a.prm.max_metrics);
        const int r = mc.advance(f);
        if (threadIdx.x == 0) {
            rqShared = r;
            if (ST) dirtyShared |= V.dirty;
        }
    }
    if (ST && a.stageMap) cp_async_wait_all();
    __syncthreads();    // the point x1 and the request are visible to the block
    const int rq = rqShared;
    if (sizeof(T) == sizeof(float) && a.x1Smem) {
        extern __shared__ float xs[];
        // the FP32 map forms alphaEff of metric and gradient points alike (a gradient point is
        // evaluated where a metric request at it would be); a gradient point also gets alpha
        // in FP64, without the conversions to float
        if (rq == REQ_F || rq == REQ_DF) {
            if (ST && a.stageMap)
                map_rows_staged<T, THREADS>(a, p, x1, rps, ec, ev, offs, tilt,
                                            reinterpret_cast<float*>(cg_smem + lay.xs), nF);
            else map_point_f32<T, THREADS>(a, p, x1, ST ? nullptr : xs);
            if (rq == REQ_DF) map_point<T, THREADS>(a, p, x1, false);
        } else if (rq == REQ_SHIFT || rq == REQ_DONE) {
            map_point<T, THREADS>(a, p, x1);
        }
    } else if (rq == REQ_F || rq == REQ_DF || rq == REQ_SHIFT) {
        map_point<T, THREADS>(a, p, x1);
    }
    if (ST) {
        // the vectors written in this round back to global memory
        const unsigned d = dirtyShared;
        for (int k = 0; k < 5; ++k)
            if ((d >> k) & 1u)
                for (int c = threadIdx.x; c < nF; c += THREADS) vg[(size_t)k * stride + c] = vb[(size_t)k * stride + c];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a.states[p] = st;
        a.req[p] = rq;
        a.gmethod[p] = st.grad_method;
        a.modeCount[p] = st.mode_count;
        if (rq != REQ_DONE) atomicAdd(a.active, 1);
        if (rq == REQ_SHIFT) atomicAdd(a.L.counters + kCounterShift, 1);
        if (rq == REQ_DF) {
            if (st.grad_method == GM_FD) a.L.fdP[atomicAdd(a.L.nFdP, 1)] = p;
            else a.L.gradP[atomicAdd(a.L.nGradP, 1)] = p;
        }
        if (a.fused && (rq == REQ_F || rq == REQ_DF)) {
            int mode = 0;
            const int refValid = ST ? tabs[0] : a.aux[2 * p + 0];
            if (rq == REQ_DF) {
                mode = 1;
                a.aux[2 * p + 0] = 1;     // the gradient pass leaves the exact object behind
            } else if (!refValid) {
                mode = 2;                 // refresh the reference object first
                a.aux[2 * p + 1] = 1;
            }
            const size_t po = (size_t)p * a.nObj;
            if (ST) enqueue_eval(a, p, rq, mode, tabs + 2, tabs + 2 + a.nObj, tabs + 2 + 2 * a.nObj, pg.chunks);
            else enqueue_eval(a, p, rq, mode, a.objCount + po, a.objFirst + po, a.objChunk0 + po, pg.chunks);
        } else if (a.phaseList && (rq == REQ_F || rq == REQ_DF)) {
            // general path with the tensor-core mode expansion: the patches to expand
            a.L.evalP[atomicAdd(a.L.nEvalP, 1)] = p;
        }
    }
    finish(rq);
}

// Re-shifts of patches that requested one (the initial re-cut of a warm start); in the solve
// rounds the solver kernel does the same for its own patch.
template <int UNUSED = 0>
__global__ void k_shift(ShiftArgs a) {
    if (a.useConditions && blockIdx.x == 0 && threadIdx.x == 0) set_round_conditions(a);
    shift_patch(a, blockIdx.x, a.req[blockIdx.x]);
}

}  // namespace rdxg
