// Size-independent kernels: per-object accumulation, the solver state machine, re-shifts.
#include "rdxg_launch.h"

namespace rdxg {

template <typename T>
void launch_accum(const KParams<T>& kp, int nPo, cudaStream_t st) {
    dim3 grid(kp.nTiles, nPo);
    k_accum<T, kAccumThreads><<<grid, kAccumThreads, 0, st>>>(kp);
}

template <typename T>
void launch_cg(const CgArgs<T>& a, int P, cudaStream_t st) {
    const size_t sm = a.x1Smem ? (size_t)a.prm.n_free * sizeof(float) : 0;
    k_cg<T, kCgThreads><<<P, kCgThreads, sm, st>>>(a);
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

template void launch_fit_plane<float>(const KParams<float>&, int, int, cudaStream_t);
template void launch_fit_plane<double>(const KParams<double>&, int, int, cudaStream_t);
template void launch_accum<float>(const KParams<float>&, int, cudaStream_t);
template void launch_accum<double>(const KParams<double>&, int, cudaStream_t);
template void launch_cg<float>(const CgArgs<float>&, int, cudaStream_t);
template void launch_cg<double>(const CgArgs<double>&, int, cudaStream_t);

}  // namespace rdxg
