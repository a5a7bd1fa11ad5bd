// Host-side launchers of the templated kernels, one explicit instantiation per
// (precision, OTF size) in rdxg_inst_<N>.cu.
#pragma once

#include <cuda_runtime.h>

#include "rdxg_cg.cuh"

namespace rdxg {

template <int N> struct Threads { static constexpr int value = (N >= 128) ? 512 : 256; };

template <typename T, int N>
struct Launcher {
    static constexpr int THREADS = Threads<N>::value;
    static size_t smem_base() { return (size_t)(Tile<N>::ELEMS + N) * sizeof(cx<T>); }
    static cudaError_t setup(int M);   // opt in to the dynamic shared memory
    static void prep(const KParams<T>& kp, int full, int nImg, cudaStream_t st);
    static void forward(const KParams<T>& kp, int nImg, cudaStream_t st);
    static void adjoint(const KParams<T>& kp, int nImg, int kind, cudaStream_t st);
    static void fd(const KParams<T>& kp, int nImg, int M, cudaStream_t st);
};

constexpr int kAccumThreads = 256;
constexpr int kCgThreads = 256;

template <typename T> void launch_accum(const KParams<T>& kp, int nPo, cudaStream_t st);
template <typename T> void launch_cg(const CgArgs<T>& a, int P, cudaStream_t st);
void launch_shift(const ShiftArgs& a, int P, cudaStream_t st);

}  // namespace rdxg
