// Issue cost of FP64 instructions against FP32 on the GPU it runs on: one warp of one block
// times 2000 iterations of four independent chains of each kind with clock64, once with all
// 32 lanes active and once with one.  Prints "<kind> <lanes> <cycles per warp instruction>".
// The per-round kernels of the solver avoid FP64 work because of these figures.
#include <cstdio>
#include <cuda_runtime.h>

__global__ void chains(double* out, long long* cycles, int kind, int oneLane, int iters) {
    const int lane = threadIdx.x & 31;
    double a = 1.0 + lane * 1e-3, a2 = a + 1, a3 = a + 2, a4 = a + 3;
    const double b = 0.999999, c = 1e-9;
    float f = 0.f;
    const long long t0 = clock64();
    if (!oneLane || lane == 0) {
        if (kind == 0) {            // DFMA
            for (int i = 0; i < iters; ++i) {
                a = fma(a, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c); a4 = fma(a4, b, c);
            }
        } else if (kind == 1) {     // double -> float conversion (the inputs step by integer adds)
            long long ia = __double_as_longlong(a), ib = __double_as_longlong(a2), ic = __double_as_longlong(a3),
                      id = __double_as_longlong(a4);
            for (int i = 0; i < iters; ++i) {
                f += (float)__longlong_as_double(ia) + (float)__longlong_as_double(ib) +
                     (float)__longlong_as_double(ic) + (float)__longlong_as_double(id);
                ia += 4096; ib += 4096; ic += 4096; id += 4096;
            }
        } else {                    // FFMA
            float x = (float)a, y = (float)a2, z = (float)a3, w = (float)a4;
            for (int i = 0; i < iters; ++i) {
                x = fmaf(x, 0.999f, 1e-9f); y = fmaf(y, 0.999f, 1e-9f); z = fmaf(z, 0.999f, 1e-9f); w = fmaf(w, 0.999f, 1e-9f);
            }
            f = x + y + z + w;
        }
    }
    __syncwarp();
    const long long t1 = clock64();
    out[threadIdx.x] = a + a2 + a3 + a4 + f;   // one value per thread of the single warp
    if (threadIdx.x == 0) *cycles = t1 - t0;
}

int main() {
    double* out = nullptr;
    long long* cyc = nullptr;
    if (cudaMalloc(&out, 32 * sizeof(double)) != cudaSuccess || cudaMalloc(&cyc, sizeof(long long)) != cudaSuccess)
        return 1;
    const char* names[3] = {"dfma", "f2f", "ffma"};
    const int iters = 2000;
    for (int kind = 0; kind < 3; ++kind)
        for (int one = 0; one < 2; ++one) {
            long long best = -1;
            for (int rep = 0; rep < 3; ++rep) {
                chains<<<1, 32>>>(out, cyc, kind, one, iters);
                long long h = 0;
                if (cudaMemcpy(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 1;
                if (best < 0 || h < best) best = h;
            }
            // four instructions of the kind per iteration (beside the conversions, FP32 adds and
            // integer adds)
            printf("%s %d %.1f\n", names[kind], one ? 1 : 32, (double)best / iters / 4);
        }
    cudaFree(out);
    cudaFree(cyc);
    return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}
