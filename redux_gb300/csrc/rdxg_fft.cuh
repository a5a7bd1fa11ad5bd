// Shared-memory 2-D FFT for one N x N complex tile per thread block.
//
// Stockham auto-sort, one radix per stage, register-staged in place: every thread loads
// the inputs of its butterflies, the block synchronises, every thread writes its outputs.
// Rows are padded to LDS = N + 1 elements so that the row pass (lanes on consecutive
// rows) and the column pass (lanes on consecutive columns) are both free of shared-memory
// bank conflicts for 8-byte elements.
//
// Convention (as FFTW): forward DIR = -1 computes X[k] = sum_x x[x] exp(-2 pi i k.x / N),
// inverse DIR = +1 the same with exp(+...), both unnormalised.
//
// Two-stage plans N = R1 * R2 (R2 may be odd: the radix-11 pass is what makes N = 88 work
// without padding, which would change the image transform).  Twiddles come from a per-N
// table tw[k] = exp(-2 pi i k / N) in shared memory, built on the host in double precision.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "fft_tables.h"

namespace rdxg {

template <typename T> struct CxT;
template <> struct CxT<float> { using type = float2; };
template <> struct CxT<double> { using type = double2; };
template <typename T> using cx = typename CxT<T>::type;

template <typename T> __device__ __forceinline__ cx<T> mkc(T r, T i) { cx<T> c; c.x = r; c.y = i; return c; }
template <typename T> __device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return mkc<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) { return mkc<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return mkc<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T> __device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
    return mkc<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T> __device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return mkc<T>(a.x * s, a.y * s); }
template <typename T> __device__ __forceinline__ T cnorm(cx<T> a) { return a.x * a.x + a.y * a.y; }
// multiply by i*s (s = +-1)
template <int S, typename T> __device__ __forceinline__ cx<T> mul_is(cx<T> a) {
    return S > 0 ? mkc<T>(-a.y, a.x) : mkc<T>(a.y, -a.x);
}

template <typename T> __device__ __forceinline__ T tab_cos(int R, int k);
template <typename T> __device__ __forceinline__ T tab_sin(int R, int k);

#define RDXG_TAB(R)                                                                                   \
    template <typename T> struct Tab##R;                                                              \
    template <> struct Tab##R<float> {                                                                \
        __device__ static __forceinline__ float c(int k) { return kCos##R##f[k]; }                    \
        __device__ static __forceinline__ float s(int k) { return kSin##R##f[k]; }                    \
    };                                                                                                \
    template <> struct Tab##R<double> {                                                               \
        __device__ static __forceinline__ double c(int k) { return kCos##R##d[k]; }                   \
        __device__ static __forceinline__ double s(int k) { return kSin##R##d[k]; }                   \
    };
RDXG_TAB(3)
RDXG_TAB(5)
RDXG_TAB(7)
RDXG_TAB(9)
RDXG_TAB(11)
RDXG_TAB(13)
RDXG_TAB(16)
#undef RDXG_TAB

template <int R, typename T> struct OddTab;
template <typename T> struct OddTab<3, T> : Tab3<T> {};
template <typename T> struct OddTab<5, T> : Tab5<T> {};
template <typename T> struct OddTab<7, T> : Tab7<T> {};
template <typename T> struct OddTab<9, T> : Tab9<T> {};
template <typename T> struct OddTab<11, T> : Tab11<T> {};
template <typename T> struct OddTab<13, T> : Tab13<T> {};

// ------------------------------ butterflies ------------------------------

template <int R, int DIR, typename T> struct Dft;

template <int DIR, typename T> struct Dft<2, DIR, T> {
    __device__ static __forceinline__ void run(cx<T>* v) {
        cx<T> a = v[0], b = v[1];
        v[0] = cadd<T>(a, b);
        v[1] = csub<T>(a, b);
    }
};

template <int DIR, typename T> struct Dft<4, DIR, T> {
    __device__ static __forceinline__ void run(cx<T>* v) {
        cx<T> a0 = cadd<T>(v[0], v[2]), a1 = csub<T>(v[0], v[2]);
        cx<T> b0 = cadd<T>(v[1], v[3]), b1 = mul_is<DIR, T>(csub<T>(v[1], v[3]));
        v[0] = cadd<T>(a0, b0);
        v[2] = csub<T>(a0, b0);
        v[1] = cadd<T>(a1, b1);
        v[3] = csub<T>(a1, b1);
    }
};

// y[u] = E[u mod H] + w^u O[u mod H], w = exp(DIR 2 pi i / R), for R = 8, 16
template <int R, int DIR, typename T> struct DftSplit {
    __device__ static __forceinline__ void run(cx<T>* v) {
        constexpr int H = R / 2;
        cx<T> e[H], o[H];
#pragma unroll
        for (int q = 0; q < H; ++q) { e[q] = v[2 * q]; o[q] = v[2 * q + 1]; }
        Dft<H, DIR, T>::run(e);
        Dft<H, DIR, T>::run(o);
#pragma unroll
        for (int u = 0; u < H; ++u) {
            // w^u = cos(2 pi u / R) + i DIR sin(2 pi u / R); table of 16ths
            constexpr int step = 16 / R;
            const T c = Tab16<T>::c(u * step);
            const T s = DIR * Tab16<T>::s(u * step);
            cx<T> t = cmul<T>(o[u], mkc<T>(c, s));
            v[u] = cadd<T>(e[u], t);
            v[u + H] = csub<T>(e[u], t);
        }
    }
};
template <int DIR, typename T> struct Dft<8, DIR, T> : DftSplit<8, DIR, T> {};
template <int DIR, typename T> struct Dft<16, DIR, T> : DftSplit<16, DIR, T> {};

// odd R: pair x[q] with x[R-q] (halves the multiplications)
template <int R, int DIR, typename T> struct DftOdd {
    __device__ static __forceinline__ void run(cx<T>* v) {
        constexpr int H = (R - 1) / 2;
        cx<T> a[H], b[H];
        cx<T> y0 = v[0];
#pragma unroll
        for (int q = 1; q <= H; ++q) {
            a[q - 1] = cadd<T>(v[q], v[R - q]);
            b[q - 1] = csub<T>(v[q], v[R - q]);
            y0 = cadd<T>(y0, a[q - 1]);
        }
        const cx<T> x0 = v[0];
        v[0] = y0;
#pragma unroll
        for (int u = 1; u <= H; ++u) {
            cx<T> A = x0, B = mkc<T>(0, 0);
#pragma unroll
            for (int q = 1; q <= H; ++q) {
                const int k = (q * u) % R;
                const T c = OddTab<R, T>::c(k), s = OddTab<R, T>::s(k);
                A.x += a[q - 1].x * c; A.y += a[q - 1].y * c;
                B.x += b[q - 1].x * s; B.y += b[q - 1].y * s;
            }
            // y[u] = A + i DIR B ; y[R-u] = A - i DIR B
            cx<T> iB = mul_is<DIR, T>(B);
            v[u] = cadd<T>(A, iB);
            v[R - u] = csub<T>(A, iB);
        }
    }
};
template <int DIR, typename T> struct Dft<3, DIR, T> : DftOdd<3, DIR, T> {};
template <int DIR, typename T> struct Dft<5, DIR, T> : DftOdd<5, DIR, T> {};
template <int DIR, typename T> struct Dft<7, DIR, T> : DftOdd<7, DIR, T> {};
template <int DIR, typename T> struct Dft<9, DIR, T> : DftOdd<9, DIR, T> {};
template <int DIR, typename T> struct Dft<11, DIR, T> : DftOdd<11, DIR, T> {};
template <int DIR, typename T> struct Dft<13, DIR, T> : DftOdd<13, DIR, T> {};

// ------------------------------ plans ------------------------------

template <int N> struct Plan;
template <> struct Plan<16> { static constexpr int R1 = 4, R2 = 4; };
template <> struct Plan<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct Plan<64> { static constexpr int R1 = 8, R2 = 8; };
template <> struct Plan<88> { static constexpr int R1 = 8, R2 = 11; };
template <> struct Plan<128> { static constexpr int R1 = 16, R2 = 8; };

// The launch-shape planner's second radix plan of each size (the first is Plan<N>): the same
// transform with the stages in the other order (or another split), which rounds differently
// and runs at a different speed.  N = 88 has none (8 * 11 is the only two-stage plan whose
// first radix is a multiple of 4, which the pruned half-plane transforms need; the
// prime-factor 11 * 8 form, without twiddle factors, was measured slower: 0.493 against
// 0.424 ms per 8100-image evaluation).
template <int N> struct PlanAlt : Plan<N> { static constexpr bool exists = false; };
template <> struct PlanAlt<32> { static constexpr int R1 = 4, R2 = 8; static constexpr bool exists = true; };
template <> struct PlanAlt<64> { static constexpr int R1 = 16, R2 = 4; static constexpr bool exists = true; };
template <> struct PlanAlt<128> { static constexpr int R1 = 8, R2 = 16; static constexpr bool exists = true; };
// plan 0: Plan<N>, plan 1: PlanAlt<N>
template <int N, int V> struct PlanOf { using type = Plan<N>; };
template <int N> struct PlanOf<N, 1> { using type = PlanAlt<N>; };

template <int N> struct Tile { static constexpr int LDS = N + 1; static constexpr int ELEMS = N * (N + 1); };

// One Stockham stage over LINES lines starting at line0.  Element e of line l is at
// s[l * lstride + e * estride].
// Thread index read through volatile asm: kernels that run several transforms inside a
// loop pass it so that the compiler cannot hoist the per-stage index arithmetic out of the
// loop (which keeps all of it live at once and spills).
__device__ __forceinline__ int opaque_tid() {
    int t;
    asm volatile("mov.u32 %0, %%tid.x;" : "=r"(t));
    return t;
}

template <typename T, int N, int R, int NS, int DIR, int LINES, int THREADS>
__device__ __forceinline__ void fft_stage(cx<T>* s, int line0, int lstride, int estride, const cx<T>* tw,
                                          int tid) {
    constexpr int BF = N / R;
    constexpr int TOTAL = LINES * BF;
    constexpr int ITER = (TOTAL + THREADS - 1) / THREADS;
    constexpr int TWS = N / (NS * R);
    cx<T> v[ITER][R];
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
        const int b = tid + it * THREADS;
        if (TOTAL % THREADS == 0 || b < TOTAL) {
            const int line = line0 + b % LINES;
            const int j = b / LINES;
            const cx<T>* base = s + line * lstride;
#pragma unroll
            for (int r = 0; r < R; ++r) v[it][r] = base[(j + r * BF) * estride];
            if (NS > 1) {
                const int k = j % NS;
#pragma unroll
                for (int r = 1; r < R; ++r) {
                    cx<T> w = tw[r * k * TWS];
                    if (DIR > 0) w.y = -w.y;
                    v[it][r] = cmul<T>(v[it][r], w);
                }
            }
            Dft<R, DIR, T>::run(v[it]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < ITER; ++it) {
        const int b = tid + it * THREADS;
        if (TOTAL % THREADS == 0 || b < TOTAL) {
            const int line = line0 + b % LINES;
            const int j = b / LINES;
            const int k = j % NS;
            const int idxD = (j / NS) * NS * R + k;
            cx<T>* base = s + line * lstride;
#pragma unroll
            for (int r = 0; r < R; ++r) base[(idxD + r * NS) * estride] = v[it][r];
        }
    }
    __syncthreads();
}

// 1-D transforms of LINES lines (rows when ROWS, else columns).
template <typename T, int N, int DIR, int LINES, bool ROWS, int THREADS, typename PL = Plan<N>>
__device__ __forceinline__ void fft_lines(cx<T>* s, int line0, const cx<T>* tw, int tid) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int R1 = PL::R1, R2 = PL::R2;
    constexpr int ls = ROWS ? LDS : 1;
    constexpr int es = ROWS ? 1 : LDS;
    fft_stage<T, N, R1, 1, DIR, LINES, THREADS>(s, line0, ls, es, tw, tid);
    fft_stage<T, N, R2, R1, DIR, LINES, THREADS>(s, line0, ls, es, tw, tid);
}

// Full 2-D transform.  IN_ROWS_PRUNED: only rows [N/4, 3N/4) of the input are non-zero
// (an n x n pupil embedded at offset n/2), so only those rows are transformed first.
template <typename T, int N, int DIR, int THREADS, bool IN_ROWS_PRUNED, typename PL = Plan<N>>
__device__ __forceinline__ void fft2d(cx<T>* s, const cx<T>* tw, int tid) {
    if (IN_ROWS_PRUNED) {
        fft_lines<T, N, DIR, N / 2, true, THREADS, PL>(s, N / 4, tw, tid);
    } else {
        fft_lines<T, N, DIR, N, true, THREADS, PL>(s, 0, tw, tid);
    }
    fft_lines<T, N, DIR, N, false, THREADS, PL>(s, 0, tw, tid);
}
template <typename T, int N, int DIR, int THREADS, bool IN_ROWS_PRUNED, typename PL = Plan<N>>
__device__ __forceinline__ void fft2d(cx<T>* s, const cx<T>* tw) {
    fft2d<T, N, DIR, THREADS, IN_ROWS_PRUNED, PL>(s, tw, (int)threadIdx.x);
}

// ---- ping-pong variant: out-of-place stages between two tiles (a -> b -> a), one barrier
// per stage and one butterfly in registers at a time ----
// RLO, RHI: only inputs r in [RLO, RHI) of each butterfly can be non-zero (the others are
// known zeros and are neither loaded nor multiplied).  The loop over a thread's butterflies is
// not unrolled: the fused evaluation keeps its accumulators in registers, and two butterflies
// in flight would spill them (measured: 0.430 ms per 8100-image evaluation against 0.479 ms
// unrolled by 2 with spills, 0.452 ms unrolled by 2 with the accumulators in shared memory).
template <typename T, int N, int R, int NS, int DIR, int LINES, int THREADS, int RLO = 0, int RHI = R>
__device__ __forceinline__ void fft_stage_pp(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst, int line0,
                                             int lstride, int estride, const cx<T>* tw) {
    constexpr int BF = N / R;
    constexpr int TOTAL = LINES * BF;
    constexpr int TWS = N / (NS * R);
#pragma unroll 1
    for (int b = threadIdx.x; b < TOTAL; b += THREADS) {
        const int line = line0 + b % LINES;
        const int j = b / LINES;
        const int k = j % NS;
        const cx<T>* in = src + line * lstride;
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = (r >= RLO && r < RHI) ? in[(j + r * BF) * estride] : mkc<T>(0, 0);
        if (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                if (r < RLO || r >= RHI) continue;
                cx<T> w = tw[r * k * TWS];
                if (DIR > 0) w.y = -w.y;
                v[r] = cmul<T>(v[r], w);
            }
        }
        Dft<R, DIR, T>::run(v);
        const int idxD = (j / NS) * NS * R + k;
        cx<T>* out = dst + line * lstride;
#pragma unroll
        for (int r = 0; r < R; ++r) out[(idxD + r * NS) * estride] = v[r];
    }
    __syncthreads();
}

// The same stage with the element loads and stores supplied by the caller: ld(line, e)
// returns element e of a line, st(line, e, v) stores output element e.  Used to fold
// element-wise work into the first or last stage of a pass.
template <typename T, int N, int R, int NS, int DIR, int LINES, int THREADS, int RLO, int RHI, typename LD,
          typename ST>
__device__ __forceinline__ void fft_stage_fn(int line0, const cx<T>* tw, LD ld, ST st) {
    constexpr int BF = N / R;
    constexpr int TOTAL = LINES * BF;
    constexpr int TWS = N / (NS * R);
#pragma unroll 1
    for (int b = threadIdx.x; b < TOTAL; b += THREADS) {
        const int line = line0 + b % LINES;
        const int j = b / LINES;
        const int k = j % NS;
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = (r >= RLO && r < RHI) ? ld(line, j + r * BF) : mkc<T>(0, 0);
        if (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                if (r < RLO || r >= RHI) continue;
                cx<T> w = tw[r * k * TWS];
                if (DIR > 0) w.y = -w.y;
                v[r] = cmul<T>(v[r], w);
            }
        }
        Dft<R, DIR, T>::run(v);
        const int idxD = (j / NS) * NS * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) st(line, idxD + r * NS, v[r]);
    }
    __syncthreads();
}

// 2-D transform in tile a (result in a), b is scratch of the same shape.
template <typename T, int N, int DIR, int THREADS, bool IN_ROWS_PRUNED, typename PL = Plan<N>>
__device__ __forceinline__ void fft2d_pp(cx<T>* a, cx<T>* b, const cx<T>* tw) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int R1 = PL::R1, R2 = PL::R2;
    constexpr int RL = IN_ROWS_PRUNED ? N / 2 : N;
    constexpr int r0 = IN_ROWS_PRUNED ? N / 4 : 0;
    fft_stage_pp<T, N, R1, 1, DIR, RL, THREADS>(a, b, r0, LDS, 1, tw);
    fft_stage_pp<T, N, R2, R1, DIR, RL, THREADS>(b, a, r0, LDS, 1, tw);
    fft_stage_pp<T, N, R1, 1, DIR, N, THREADS>(a, b, 0, 1, LDS, tw);
    fft_stage_pp<T, N, R2, R1, DIR, N, THREADS>(b, a, 0, 1, LDS, tw);
}

// ping-pong transform whose output is only needed on rows [N/4, 3N/4): columns first
template <typename T, int N, int DIR, int THREADS, typename PL = Plan<N>>
__device__ __forceinline__ void fft2d_pp_out_rows_pruned(cx<T>* a, cx<T>* b, const cx<T>* tw) {
    constexpr int LDS = Tile<N>::LDS;
    constexpr int R1 = PL::R1, R2 = PL::R2;
    fft_stage_pp<T, N, R1, 1, DIR, N, THREADS>(a, b, 0, 1, LDS, tw);
    fft_stage_pp<T, N, R2, R1, DIR, N, THREADS>(b, a, 0, 1, LDS, tw);
    fft_stage_pp<T, N, R1, 1, DIR, N / 2, THREADS>(a, b, N / 4, LDS, 1, tw);
    fft_stage_pp<T, N, R2, R1, DIR, N / 2, THREADS>(b, a, N / 4, LDS, 1, tw);
}

// Two tiles of FP32 fit in shared memory up to N = 88: kernels that loop over work items
// use the ping-pong transforms there (no register staging, nothing to hoist out of loops).
template <typename T, int N> struct PingPong {
    static constexpr bool value = sizeof(T) == 4 && N <= 88;
};

template <typename T, int N, int DIR, int THREADS, bool IN_ROWS_PRUNED>
__device__ __forceinline__ void fft2d_any(cx<T>* a, cx<T>* b, const cx<T>* tw) {
    if constexpr (PingPong<T, N>::value) fft2d_pp<T, N, DIR, THREADS, IN_ROWS_PRUNED>(a, b, tw);
    else fft2d<T, N, DIR, THREADS, IN_ROWS_PRUNED>(a, tw);
}

// 2-D transform whose output is only needed on rows [N/4, 3N/4): columns first, then the
// needed rows.
template <typename T, int N, int DIR, int THREADS, typename PL = Plan<N>>
__device__ __forceinline__ void fft2d_out_rows_pruned(cx<T>* s, const cx<T>* tw, int tid) {
    fft_lines<T, N, DIR, N, false, THREADS, PL>(s, 0, tw, tid);
    fft_lines<T, N, DIR, N / 2, true, THREADS, PL>(s, N / 4, tw, tid);
}
template <typename T, int N, int DIR, int THREADS, typename PL = Plan<N>>
__device__ __forceinline__ void fft2d_out_rows_pruned(cx<T>* s, const cx<T>* tw) {
    fft2d_out_rows_pruned<T, N, DIR, THREADS, PL>(s, tw, (int)threadIdx.x);
}

}  // namespace rdxg
