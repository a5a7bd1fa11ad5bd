// Size-independent kernels: per-object accumulation, the solver state machine, re-shifts.
#include "rdxg_launch.h"

namespace rdxg {

template <typename T>
void launch_accum(const KParams<T>& kp, int nPo, cudaStream_t st) {
    dim3 grid(kp.nTiles, nPo);
    k_accum<T, kAccumThreads><<<grid, kAccumThreads, 0, st>>>(kp);
}

template <typename T>
void launch_cg(const CgArgs<T>& a, const ShiftArgs& sa, int P, cudaStream_t st) {
    if (a.stage) {
        const int nT = a.fused ? a.nTilesH : a.nTiles;
        const size_t sm = CgStageLayout(a.prm.n_free, a.nObj, nT, a.stageMap, a.nPar, a.I, a.maxNnz).total;
        k_cg<T, kCgThreads, true><<<P, kCgThreads, sm, st>>>(a, sa);
        return;
    }
    const size_t sm = a.x1Smem ? (size_t)a.prm.n_free * sizeof(float) : 0;
    k_cg<T, kCgThreads, false><<<P, kCgThreads, sm, st>>>(a, sa);
}

template <typename T>
cudaError_t setup_cg(size_t stageBytes) {
    return raise_smem_limit(k_cg<T, kCgThreads, true>, stageBytes);
}

__global__ void k_to_float(const double* src, float* dst, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = (float)src[i];
}
void launch_to_float(const double* src, float* dst, size_t n, cudaStream_t st) {
    const size_t blocks = (n + 255) / 256;
    if (blocks) k_to_float<<<(int)(blocks < 4096 ? blocks : 4096), 256, 0, st>>>(src, dst, n);
}

void launch_shift(const ShiftArgs& a, int P, cudaStream_t st) {
    k_shift<0><<<P, 128, 0, st>>>(a);
}

template <typename T>
void launch_fit_plane(const KParams<T>& kp, int full, int nPo, cudaStream_t st) {
    k_fit_plane<T, 256><<<nPo, 256, 0, st>>>(kp, full);
}

void launch_add_plane(const double* plane, float* objects, int nPo, int ps, cudaStream_t st) {
    k_add_plane<0><<<nPo, 256, 0, st>>>(plane, objects, ps);
}

// End of one iteration of the solve graph's device loop: the loop (a WHILE node) continues
// while any handle has an active patch, for at most maxRounds rounds in all.  One thread.
__global__ void k_loop_cond(LoopArgs a) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    int any = 0;
    for (int k = 0; k < a.nActive; ++k) any |= (*a.active[k] != 0);
    const long long r = (*a.rounds += a.roundsPerIteration);
    *a.launchCount += 1ull;
    if (any && r > a.maxRounds) {
        *a.overrun = 1;
        any = 0;
    }
    cudaGraphSetConditional(a.loop, any ? 1u : 0u);
}

void launch_loop_cond(const LoopArgs& a, cudaStream_t st) { k_loop_cond<<<1, 32, 0, st>>>(a); }

// %nsmid: one more than the largest SM identifier %smid can hold (identifiers need not be
// contiguous), the size of the per-SM slot masks of the recomputing kernels
__global__ void k_nsmid(int32_t* out) {
    unsigned v;
    asm volatile("mov.u32 %0, %%nsmid;" : "=r"(v));
    if (threadIdx.x == 0) *out = (int32_t)v;
}

cudaError_t query_nsmid(int32_t* dOut, int32_t* hOut, cudaStream_t st) {
    k_nsmid<<<1, 32, 0, st>>>(dOut);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hOut, dOut, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e;
}

template void launch_fit_plane<float>(const KParams<float>&, int, int, cudaStream_t);
template void launch_fit_plane<double>(const KParams<double>&, int, int, cudaStream_t);
template void launch_accum<float>(const KParams<float>&, int, cudaStream_t);
template void launch_accum<double>(const KParams<double>&, int, cudaStream_t);
template void launch_cg<float>(const CgArgs<float>&, const ShiftArgs&, int, cudaStream_t);
template void launch_cg<double>(const CgArgs<double>&, const ShiftArgs&, int, cudaStream_t);
template cudaError_t setup_cg<float>(size_t);
template cudaError_t setup_cg<double>(size_t);

}  // namespace rdxg
