// Definitions of Launcher<T, N>; included once per OTF size by rdxg_inst_<N>.cu.
#pragma once

#include "rdxg_launch.h"

namespace rdxg {

template <typename T, int N>
static size_t extra_smem(int M) {
    size_t a = (size_t)M * sizeof(T);
    size_t b = (size_t)(N / 2) * (N / 2) * sizeof(T);
    size_t c = 33 * sizeof(double);
    size_t m = a > b ? a : b;
    return (m > c ? m : c) + 16;
}

template <typename T, int N>
cudaError_t Launcher<T, N>::setup(int M) {
    const int sm = (int)(smem_base() + extra_smem<T, N>(M));
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_prep<T, N, THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))) return e;
    if ((e = cudaFuncSetAttribute(k_forward<T, N, THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))) return e;
    if ((e = cudaFuncSetAttribute(k_adjoint<T, N, THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))) return e;
    if ((e = cudaFuncSetAttribute(k_fd<T, N, THREADS>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm))) return e;
    return cudaSuccess;
}

template <typename T, int N>
void Launcher<T, N>::prep(const KParams<T>& kp, int full, int nImg, cudaStream_t st) {
    const size_t sm = smem_base() + extra_smem<T, N>(kp.M);
    k_prep<T, N, THREADS><<<nImg, THREADS, sm, st>>>(kp, full);
}

template <typename T, int N>
void Launcher<T, N>::forward(const KParams<T>& kp, int nImg, cudaStream_t st) {
    const size_t sm = smem_base() + extra_smem<T, N>(kp.M);
    k_forward<T, N, THREADS><<<nImg, THREADS, sm, st>>>(kp);
}

template <typename T, int N>
void Launcher<T, N>::adjoint(const KParams<T>& kp, int nImg, int kind, cudaStream_t st) {
    const size_t sm = smem_base() + extra_smem<T, N>(kp.M);
    k_adjoint<T, N, THREADS><<<nImg, THREADS, sm, st>>>(kp, kind);
}

template <typename T, int N>
void Launcher<T, N>::fd(const KParams<T>& kp, int nImg, int M, cudaStream_t st) {
    const size_t sm = smem_base() + extra_smem<T, N>(kp.M);
    dim3 grid(nImg, M);
    k_fd<T, N, THREADS><<<grid, THREADS, sm, st>>>(kp);
}

}  // namespace rdxg
