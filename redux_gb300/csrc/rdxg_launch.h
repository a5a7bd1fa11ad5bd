// Host-side launchers of the templated kernels, one explicit instantiation per
// (precision, OTF size) in rdxg_inst_<N>.cu.
#pragma once

#include <cuda_runtime.h>

#include <mutex>

#include "rdxg_cg.cuh"
#include "rdxg_restore.cuh"

namespace rdxg {

// Raises a kernel's dynamic shared memory limit to at least `bytes`, never lowering it: the
// attribute belongs to the function for the whole process, so every handle (of any geometry)
// shares it, and one set by a handle with smaller needs must not break another's launches.
inline std::mutex& smem_limit_mutex() {
    static std::mutex m;
    return m;
}
template <typename K>
cudaError_t raise_smem_limit(K* kernel, size_t bytes) {
    std::lock_guard<std::mutex> lock(smem_limit_mutex());
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kernel);
    if (e != cudaSuccess) return e;
    if ((size_t)fa.maxDynamicSharedSizeBytes >= bytes) return cudaSuccess;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

template <int N> struct Threads { static constexpr int value = (N >= 128) ? 512 : 256; };
// The alternative block size of the one-image-per-block kernels (k_forward, k_adjoint) in
// FP32, picked by the launch-shape planner when it measures faster: the per-element
// arithmetic does not depend on the block size, so neither do the results.
template <int N> struct ThreadsAlt { static constexpr int value = 2 * Threads<N>::value; };

template <typename T, int N>
struct Launcher {
    static constexpr int THREADS = Threads<N>::value;
    // the work tile (unless it lives in global memory, GlobalTile) and the twiddles
    static size_t smem_base() {
        return (size_t)((GlobalTile<T, N>::value ? 0 : Tile<N>::ELEMS) + N) * sizeof(cx<T>);
    }
    static cudaError_t setup(int M);   // opt in to the dynamic shared memory
    static void prep(const KParams<T>& kp, int full, int nImg, cudaStream_t st);
    static void forward(const KParams<T>& kp, int nImg, cudaStream_t st);
    static void adjoint(const KParams<T>& kp, int grid, int kind, cudaStream_t st);   // grid-strides over the work list
    static void fd(const KParams<T>& kp, int grid, int M, cudaStream_t st);
    // resident blocks per SM of the kernels that recompute the transforms (the scratch slots
    // per SM), 0 when their shared memory does not fit
    static int recompute_occupancy(int M);
    static cudaError_t restore(const KParams<T>& kp, const RestoreArgs& ra, int nBlocks, cudaStream_t st);
    // PSF / convolved-object / residual outputs after restore(); grid: blocks (each with its
    // 3 N^2 doubles of oa.pool)
    static cudaError_t restore_outputs(const KParams<T>& kp, const RestoreOutArgs& oa, int grid, cudaStream_t st);
};

constexpr int kAccumThreads = 256;
constexpr int kCgThreads = 256;

template <typename T> void launch_accum(const KParams<T>& kp, int nPo, cudaStream_t st);
// FIT_PLANE: fit the planes of every (patch, object) (full) or of those with a re-initialised
// image, and add them to the restored objects
template <typename T> void launch_fit_plane(const KParams<T>& kp, int full, int nPo, cudaStream_t st);
void launch_add_plane(const double* plane, float* objects, int nPo, int ps, cudaStream_t st);

// fused evaluation (FP32, N <= 88): block size of k_eval and k_fd_half (a multiple of 32;
// the transform stages stride over any size)
#ifndef RDXG_EVAL_THREADS
#define RDXG_EVAL_THREADS 512
#endif
constexpr int kEvalThreads = RDXG_EVAL_THREADS;
static_assert(kEvalThreads % 32 == 0 && kEvalThreads <= 1024, "block size");
// the planner's alternative block size of k_eval (results are the same: each half-plane
// point is accumulated by one thread, whatever the block size)
constexpr int kEvalThreadsAlt = kEvalThreads == 384 ? 512 : 384;
constexpr int kReduceThreads = 256;
constexpr int kPhasePix = 256;      // pixels per block of the mode expansion
constexpr int kMaxChunk = 32;       // images per chunk (upper bound)
constexpr int kPhaseRegPix = 128;   // pixels per block of the per-patch mode expansion
constexpr int kPhaseRegModes = 64;  // modes it holds in registers (more: the staged kernel)
constexpr int kPhaseMaxImg = 64;    // images per patch it stages
constexpr int kPhaseMaxCh = 16;     // channels whose fixed phases it stages
constexpr int kNumCounters = 9;     // work-list counters reset every round (and the evaluation's two)
constexpr size_t kMaxSmem = 227 * 1024;   // dynamic shared memory per block
template <typename T, int N> struct EvalLauncher {
    static cudaError_t setup(int M, int npt, int nH);
    static void eval(const EvalParams<T>& e, int npt, int grid, cudaStream_t st);
    static void reduce(const EvalParams<T>& e, int grid, cudaStream_t st);
    static void phase(const EvalParams<T>& e, int grid, cudaStream_t st);
    static size_t smem(int M, int nH);
    static int occupancy(int M, int npt, int nH);   // resident blocks per SM
    static int phase_tiles();                        // pixel tiles of the per-patch mode expansion
    static size_t fd_smem(int nH);                   // shared memory of the half-plane FD gradient
    static void fd_half(const EvalParams<T>& e, int grid, cudaStream_t st);
};
template <typename T> void launch_cg(const CgArgs<T>& a, const ShiftArgs& sa, int P, cudaStream_t st);
constexpr size_t kCgStageBytes = 96 * 1024;   // shared memory of the staged solver kernel, at most
template <typename T> cudaError_t setup_cg(size_t stageBytes);   // opt in to it
cudaError_t query_nsmid(int32_t* dOut, int32_t* hOut, cudaStream_t st);   // %nsmid of the device
void launch_shift(const ShiftArgs& a, int P, cudaStream_t st);
void launch_to_float(const double* src, float* dst, size_t n, cudaStream_t st);   // dst = (float)src

// The device loop of a solve graph: a WHILE node whose body runs roundsPerIteration rounds of
// every handle and then k_loop_cond, which keeps the loop going while a handle has an active
// patch (bounded by maxRounds; past it, *overrun is set and the loop ends).
struct LoopArgs {
    cudaGraphConditionalHandle loop;
    int32_t* const* active;      // [nActive] each handle's active-patch counter
    int32_t nActive;
    int32_t roundsPerIteration;
    long long maxRounds;
    long long* rounds;           // rounds run so far (zeroed before the graph launch)
    int32_t* overrun;
    unsigned long long* launchCount;
};
void launch_loop_cond(const LoopArgs& a, cudaStream_t st);

// mode expansion on the tensor cores (rdxg_phase_tc.cu); parts: 2 (3xBF16) or 3 (6xBF16)
PhaseTcPlan phase_tc_plan(int I, int M, int n2, int nCh, int parts, int numSMs);
void launch_tc_pack_modes(const float* Z, const float* phiFixed, int M, int C, int n2, const PhaseTcPlan& p,
                          __nv_bfloat16* out, cudaStream_t st);
void launch_phase_tc(const PhaseTcArgs& a, const PhaseTcPlan& p, cudaStream_t st);

// rdxg_metric_noalloc: a fixed static device array holds every temporary of the evaluation
constexpr size_t kNoAllocScratchBytes = (size_t)16 << 20;
cudaError_t noalloc_scratch(void** ptr);   // its address in the current context (loads the module)
void launch_noalloc_alpha(const double* alpha, const double* curTilt, const double* resAlpha, int G, int M,
                          int tiltX, int tiltY, float* alphaEff, cudaStream_t st);
void launch_noalloc_lists(int P, int nObj, const int32_t* objFirst, const int32_t* objCount, const int32_t* objChunk0,
                          int chunkSize, int chunksPerPatch, int mode, const Lists& L, cudaStream_t st);
void launch_noalloc_metric(const double* objMetric, int P, int nObj, int nTiles, const double* objWeight, double ps2,
                           double* metric, cudaStream_t st);

}  // namespace rdxg
