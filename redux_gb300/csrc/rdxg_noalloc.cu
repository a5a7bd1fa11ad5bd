// Static scratch and helper kernels of rdxg_metric_noalloc: the metric evaluation with every
// temporary in one file-scope device array instead of buffers of the handle.
#include "rdxg_launch.h"

namespace rdxg {

// The scratch itself: part of the module's global memory, set up when the module is loaded,
// never allocated or freed by a call.  Shared by every handle on a device, so calls that use
// it must not overlap.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

cudaError_t noalloc_scratch(void** ptr) {
    // The address in the current context.  Looking it up also loads this file's module if the
    // runtime loads modules lazily, which is when the array's memory is reserved: rdxg_create
    // calls this, so that reservation happens when the handle is made, not in a later call.
    *ptr = nullptr;
    return cudaGetSymbolAddress(ptr, g_noalloc_scratch);
}

// alphaEff = alpha with the tilt modes moved by the current tilt offset minus the residual
// tilt, as the host does for rdxg_metric (same double arithmetic, then rounded to float).
__global__ void k_noalloc_alpha(const double* alpha, const double* curTilt, const double* resAlpha, int G, int M,
                                int tiltX, int tiltY, float* alphaEff) {
    const size_t n = (size_t)G * M;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t g = i / M;
        const int m = (int)(i % M);
        double v = alpha[i];
        if (m == tiltX) v += curTilt[g * 2 + 1] - resAlpha[g * 2 + 1];
        else if (m == tiltY) v += curTilt[g * 2 + 0] - resAlpha[g * 2 + 0];
        alphaEff[i] = (float)v;
    }
}

// Work lists of one evaluation of every patch, in the order the host builds them for
// rdxg_metric: patch by patch, object by object, chunk by chunk.  One thread per patch.
__global__ void k_noalloc_lists(int P, int nObj, const int32_t* objFirst, const int32_t* objCount,
                                const int32_t* objChunk0, int chunkSize, int chunksPerPatch, int mode, Lists L) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p == 0) {
        L.nEval[0] = P * chunksPerPatch;
        *L.nPo = P * nObj;
        *L.nEvalP = P;
    }
    if (p >= P) return;
    L.evalP[p] = p;
    for (int o = 0; o < nObj; ++o) {
        const int cnt = objCount[o];
        const int nc = (cnt + chunkSize - 1) / chunkSize;
        for (int c = 0; c < nc; ++c) {
            EvalItem it;
            it.p = p; it.o = o;
            it.first = objFirst[o] + c * chunkSize;
            it.count = min(chunkSize, cnt - c * chunkSize);
            it.chunk = objChunk0[o] + c;
            it.df = 0;
            L.eval[(size_t)p * chunksPerPatch + objChunk0[o] + c] = it;
        }
        PoItem pi;
        pi.p = p; pi.o = o; pi.mode = mode;
        L.po[(size_t)p * nObj + o] = pi;
    }
}

// metric[p] = sum_o w_o * (sum_t tile[p][o][t]) / ps^2, tiles and objects in order (the
// host's summation for rdxg_metric); one thread per patch.
__global__ void k_noalloc_metric(const double* objMetric, int P, int nObj, int nTiles, const double* objWeight,
                                 double ps2, double* metric) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= P) return;
    double sum = 0;
    for (int o = 0; o < nObj; ++o) {
        const double w = objWeight[o];
        if (w == 0.0) continue;
        double m = 0;
        const double* t = objMetric + ((size_t)p * nObj + o) * nTiles;
        for (int k = 0; k < nTiles; ++k) m = __dadd_rn(m, t[k]);
        sum = __dadd_rn(sum, __dmul_rn(w, __ddiv_rn(m, ps2)));
    }
    metric[p] = sum;
}

void launch_noalloc_alpha(const double* alpha, const double* curTilt, const double* resAlpha, int G, int M,
                          int tiltX, int tiltY, float* alphaEff, cudaStream_t st) {
    k_noalloc_alpha<<<256, 256, 0, st>>>(alpha, curTilt, resAlpha, G, M, tiltX, tiltY, alphaEff);
}

void launch_noalloc_lists(int P, int nObj, const int32_t* objFirst, const int32_t* objCount, const int32_t* objChunk0,
                          int chunkSize, int chunksPerPatch, int mode, const Lists& L, cudaStream_t st) {
    k_noalloc_lists<<<(P + 127) / 128, 128, 0, st>>>(P, nObj, objFirst, objCount, objChunk0, chunkSize,
                                                      chunksPerPatch, mode, L);
}

void launch_noalloc_metric(const double* objMetric, int P, int nObj, int nTiles, const double* objWeight, double ps2,
                           double* metric, cudaStream_t st) {
    k_noalloc_metric<<<(P + 127) / 128, 128, 0, st>>>(objMetric, P, nObj, nTiles, objWeight, ps2, metric);
}

}  // namespace rdxg
