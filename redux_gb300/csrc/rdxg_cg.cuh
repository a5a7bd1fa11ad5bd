// Device side of the per-patch optimiser: one thread block per patch runs the state
// machine of cg_machine.h (scalar logic replicated in every thread, vector operations
// block-parallel, all sums in double in a fixed order), maps the point of the next
// evaluation through the null-space map (Constraints::reverseAndAdd,
// constraints.hpp:141-146) and the gradient back (Constraints::apply, 128-133), and
// performs the integer image re-shifts between mode stages (SubImage::adjustShifts,
// subimage.cpp:444-480).
#pragma once

#include "cg_machine.h"
#include "rdxg_eval.cuh"
#include "rdxg_kernels.cuh"

namespace rdxg {

template <int THREADS>
struct DevVec {
    int n;
    double* red;
    __device__ void copy(double* d, const double* s) {
        for (int i = threadIdx.x; i < n; i += THREADS) d[i] = s[i];
        __syncthreads();
    }
    __device__ void zero(double* d) {
        for (int i = threadIdx.x; i < n; i += THREADS) d[i] = 0.0;
        __syncthreads();
    }
    __device__ double nrm2(const double* v) {
        double a = 0;
        for (int i = threadIdx.x; i < n; i += THREADS) a += v[i] * v[i];
        return sqrt(block_sum<THREADS>(a, red));
    }
    __device__ double dot(const double* x, const double* y) {
        double a = 0;
        for (int i = threadIdx.x; i < n; i += THREADS) a += x[i] * y[i];
        return block_sum<THREADS>(a, red);
    }
    __device__ double pr_update(double* g0, const double* g) {
        double a = 0;
        for (int i = threadIdx.x; i < n; i += THREADS) {
            const double t = g0[i] - g[i];
            a += t * g[i];
            g0[i] = t;
        }
        return block_sum<THREADS>(a, red);
    }
    __device__ void dir_update(double* p, const double* g, double beta) {
        for (int i = threadIdx.x; i < n; i += THREADS) p[i] = g[i] - beta * p[i];
        __syncthreads();
    }
    __device__ void step(double* x1, const double* x, const double* p, double s) {
        for (int i = threadIdx.x; i < n; i += THREADS) x1[i] = x[i] + s * p[i];
        __syncthreads();
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
    const double* galpha;   // [P][nPar]
    const double* partial;  // [P][nObj][nTiles]
    const double* objWeight;
    // null-space map, by parameter row and by free column
    const int32_t* rowPtr; const int32_t* rowCol; const double* rowVal;
    const float* rowVal32;  // FP32 copy of rowVal
    int32_t x1Smem;         // FP32 metric-request map enabled (dynamic shared memory n_free floats)
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
    const int32_t* objChunk0;      // [nObj]
    const int32_t* objFirst;       // [nObj]
    const int32_t* objCount;       // [nObj]
    int32_t* aux;                  // [P][2]: reference object valid, refresh pending
};

// alpha = offset + N x1; alpha_eff = alpha + currentTiltOffset - residual for the tilt modes
// (the residual is what Channel::initPatch adds to phi_channel, channel.cpp:916-939)
template <typename T, int THREADS>
__device__ void map_point(const CgArgs<T>& a, int p, const double* x1) {
    const double* off = a.alphaOff + (size_t)p * a.nPar;
    double* al = a.alpha + (size_t)p * a.nPar;
    T* ae = a.alphaEff + (size_t)p * a.nPar;
    for (int r = threadIdx.x; r < a.nPar; r += THREADS) {
        double v = off[r];
        for (int e = a.rowPtr[r]; e < a.rowPtr[r + 1]; ++e) v += a.rowVal[e] * x1[a.rowCol[e]];
        al[r] = v;
        const int j = r / a.M, m = r % a.M;
        double ve = v;
        const size_t b = ((size_t)p * a.I + j) * 2;
        if (m == a.tiltX) ve += a.curTilt[b + 1] - a.resAlpha[b + 1];
        else if (m == a.tiltY) ve += a.curTilt[b + 0] - a.resAlpha[b + 0];
        ae[r] = (T)ve;
    }
    __syncthreads();
}

// The FP32 path's metric requests: alphaEff only, in FP32 arithmetic (it is rounded to FP32
// for the evaluation anyway), with the point staged in shared memory as float.  GB300's FP64
// rate makes the FP64 map the largest cost of the solver kernel; the FP64 alpha is formed by
// map_point for every gradient, re-shift and final point, where it is used.
template <typename T, int THREADS>
__device__ void map_point_f32(const CgArgs<T>& a, int p, const double* x1, float* xs) {
    const int nF = a.prm.n_free;
    for (int c = threadIdx.x; c < nF; c += THREADS) xs[c] = (float)x1[c];
    __syncthreads();
    const double* off = a.alphaOff + (size_t)p * a.nPar;
    T* ae = a.alphaEff + (size_t)p * a.nPar;
    for (int r = threadIdx.x; r < a.nPar; r += THREADS) {
        float v = 0.f;
        for (int e = a.rowPtr[r]; e < a.rowPtr[r + 1]; ++e) v = fmaf(a.rowVal32[e], xs[a.rowCol[e]], v);
        v += (float)off[r];
        const int j = r / a.M, m = r % a.M;
        const size_t b = ((size_t)p * a.I + j) * 2;
        if (m == a.tiltX) v += (float)(a.curTilt[b + 1] - a.resAlpha[b + 1]);
        else if (m == a.tiltY) v += (float)(a.curTilt[b + 0] - a.resAlpha[b + 0]);
        ae[r] = (T)v;
    }
    __syncthreads();
}

// append the chunks and objects of patch p to the evaluation work lists
template <typename T>
__device__ void enqueue_eval(const CgArgs<T>& a, int p, int rq, int mode) {
    a.L.evalP[atomicAdd(a.L.nEvalP, 1)] = p;
    for (int o = 0; o < a.nObj; ++o) {
        const int cnt = a.objCount[o];
        const int nc = (cnt + a.chunkSize - 1) / a.chunkSize;
        for (int c = 0; c < nc; ++c) {
            EvalItem it;
            it.p = p; it.o = o;
            it.first = a.objFirst[o] + c * a.chunkSize;
            it.count = min(a.chunkSize, cnt - c * a.chunkSize);
            it.chunk = a.objChunk0[o] + c;
            it.df = (rq == REQ_DF) ? 1 : 0;
            const int k = atomicAdd(a.L.nEval, 1);
            a.L.eval[k] = it;
        }
        PoItem pi;
        pi.p = p; pi.o = o; pi.mode = mode;
        const int k = atomicAdd(a.L.nPo, 1);
        a.L.po[k] = pi;
    }
}

template <typename T, int THREADS>
__global__ void __launch_bounds__(THREADS) k_cg(CgArgs<T> a) {
    const int p = blockIdx.x;
    __shared__ double red[33];
    __shared__ double fsh;
    CgState st = a.states[p];
    const int nF = a.prm.n_free;
    double* x = a.vec + (size_t)p * 5 * nF;
    double* pv = x + nF;
    double* g = pv + nF;
    double* g0 = g + nF;
    double* x1 = g0 + nF;
    if (st.pc == PC_DONE) {
        if (threadIdx.x == 0) a.req[p] = REQ_DONE;
        return;
    }
    double f = 0;
    if (a.fused && st.req == REQ_F && a.aux[2 * p + 1]) {
        // the last evaluation only refreshed the reference object: repeat the request
        __syncthreads();
        if (threadIdx.x == 0) {
            a.aux[2 * p + 0] = 1;
            a.aux[2 * p + 1] = 0;
            a.req[p] = REQ_F;
            atomicAdd(a.active, 1);
            enqueue_eval(a, p, REQ_F, 0);
        }
        return;
    }
    if (st.req == REQ_F) {
        // the block loads the per-tile sums of the patch's objects in parallel; thread 0
        // adds them tile by tile, object by object, in a fixed order
        __shared__ double tiles[THREADS];
        const int nT = a.fused ? a.nTilesH : a.nTiles;
        const double* src = (a.fused ? a.objMetric : a.partial) + (size_t)p * a.nObj * nT;
        const int total = a.nObj * nT;
        double sum = 0, m = 0;
        for (int base = 0; base < total; base += THREADS) {
            const int i = base + threadIdx.x;
            tiles[threadIdx.x] = i < total ? src[i] : 0.0;
            __syncthreads();
            if (threadIdx.x == 0) {
                const int cnt = min(THREADS, total - base);
                for (int k = 0; k < cnt; ++k) {
                    const int o = (base + k) / nT, t = (base + k) % nT;
                    m += tiles[k];
                    if (t == nT - 1) {
                        const double w = a.objWeight[o];
                        if (w != 0.0) sum += w * (m / ((double)a.ps * a.ps));
                        m = 0;
                    }
                }
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) fsh = sum;
        __syncthreads();
        f = fsh;
    } else if (st.req == REQ_DF) {
        const double* ga = a.galpha + (size_t)p * a.nPar;
        for (int c = threadIdx.x; c < nF; c += THREADS) {
            double v = 0;
            for (int e = a.colPtr[c]; e < a.colPtr[c + 1]; ++e) v += a.colVal[e] * ga[a.colRow[e]];
            g[c] = v;
        }
        __syncthreads();
    } else if (st.req == REQ_SHIFT) {
        double* off = a.alphaOff + (size_t)p * a.nPar;
        const double* al = a.alpha + (size_t)p * a.nPar;
        for (int r = threadIdx.x; r < a.nPar; r += THREADS) off[r] = al[r];
        __syncthreads();
    }
    DevVec<THREADS> V{nF, red};
    Machine<DevVec<THREADS>> mc(a.prm, st, V, x, pv, g, g0, x1, a.metrics + (size_t)p * a.prm.max_metrics);
    const int rq = mc.advance(f);
    if (sizeof(T) == sizeof(float) && a.x1Smem) {
        extern __shared__ float xs[];
        if (rq == REQ_F) map_point_f32<T, THREADS>(a, p, x1, xs);
        else if (rq == REQ_DF || rq == REQ_SHIFT || rq == REQ_DONE) map_point<T, THREADS>(a, p, x1);
    } else if (rq == REQ_F || rq == REQ_DF || rq == REQ_SHIFT) {
        map_point<T, THREADS>(a, p, x1);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a.states[p] = st;
        a.req[p] = rq;
        a.gmethod[p] = st.grad_method;
        a.modeCount[p] = st.mode_count;
        if (rq != REQ_DONE) atomicAdd(a.active, 1);
        if (rq == REQ_DF) {
            if (st.grad_method == GM_FD) a.L.fdP[atomicAdd(a.L.nFdP, 1)] = p;
            else a.L.gradP[atomicAdd(a.L.nGradP, 1)] = p;
        }
        if (a.fused && (rq == REQ_F || rq == REQ_DF)) {
            int mode = 0;
            if (rq == REQ_DF) {
                mode = 1;
                a.aux[2 * p + 0] = 1;     // the gradient pass leaves the exact object behind
            } else if (!a.aux[2 * p + 0]) {
                mode = 2;                 // refresh the reference object first
                a.aux[2 * p + 1] = 1;
            }
            enqueue_eval(a, p, rq, mode);
        }
    }
}

// adjustShifts for every image of patches that requested a re-shift; marks the images of
// every object that has a shifted image for re-initialisation (Object::reInitialize).
struct ShiftArgs {
    int32_t P, I, M, nObj, ps, cs, margin, tiltX, tiltY;
    const int32_t* req;
    const double* alpha;     // [P][I*M]
    double* tiltOff;         // [P][I][2] currentTiltOffset (y, x)
    int32_t* shift;          // [P][I][2]
    uint8_t* reinit;         // [P][I]
    const int32_t* imgObj;
    int32_t* aux;            // [P][2] reference object valid flag (cleared on re-initialisation)
    double J[2][2], Jinv[2][2];
};

template <int UNUSED = 0>
__global__ void k_shift(ShiftArgs a) {
    const int p = blockIdx.x;
    if (a.req[p] != REQ_SHIFT) {
        for (int j = threadIdx.x; j < a.I; j += blockDim.x) a.reinit[(size_t)p * a.I + j] = 0;
        return;
    }
    __shared__ int objShifted[64];
    for (int o = threadIdx.x; o < a.nObj; o += blockDim.x) objShifted[o] = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < a.I; j += blockDim.x) {
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
            atomicExch(&objShifted[a.imgObj[j]], 1);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < a.I; j += blockDim.x) {
        const int sh = objShifted[a.imgObj[j]];
        a.reinit[(size_t)p * a.I + j] = sh ? 1 : 0;
        if (sh && a.aux) a.aux[2 * p + 0] = 0;
    }
}

}  // namespace rdxg
