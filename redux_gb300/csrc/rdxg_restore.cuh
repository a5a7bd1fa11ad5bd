// Restoration of the objects of every patch: Object::restorePatch (object.cpp:278-334) for
// the restored object, with SubImage::restore (subimage.cpp:242-256) and ScharmerFilter,
// smooth and connectedRegion (image/utils.cpp:49-57, 295-392).  FP64 throughout (the image
// transforms and OTFs enter as stored, FP32 or FP64): one block per (patch, object), the
// N x N work arrays in global scratch, the final inverse transform in shared memory.
#pragma once

#include "rdxg_kernels.cuh"

namespace rdxg {

struct RestoreArgs {
    const double* fc;      // [nObj] Object::frequencyCutoff (the filter uses 0.9 of it)
    int32_t noFilter;      // RF_NO_FILTER
    double* scratch;       // [P * nObj][kRestoreScratch * N * N]
    float* out;            // [P][nObj][ps][ps]
};
constexpr int kRestoreScratch = 7;   // doubles per frequency: object (2), den, pt, rr, tmp, mask
constexpr int kRestoreBand = 16;     // lines per band of the final inverse transform

// smooth (utils.cpp:304-328): mean over [y-nY, y+nY) x [x-nX, x+nX) clipped to the array, the
// sum in the reference's order
template <int N, int THREADS>
__device__ __forceinline__ void restore_smooth(const double* in, double* out, int nY, int nX) {
    for (int c = threadIdx.x; c < N * N; c += THREADS) {
        const int y = c / N, x = c % N;
        const int yl = max(y - nY, 0), yh = min(y + nY, N), xl = max(x - nX, 0), xh = min(x + nX, N);
        double t = 0;
        int cnt = 0;
        for (int yy = yl; yy < yh; ++yy)
            for (int xx = xl; xx < xh; ++xx) { t += in[yy * N + xx]; cnt++; }
        out[c] = t / cnt;
    }
    __syncthreads();
}

template <typename T, int N, int THREADS>
__global__ void __launch_bounds__(THREADS) k_restore(KParams<T> kp, RestoreArgs ra) {
    constexpr int N2 = N * N, LDS = Tile<N>::LDS;
    const int b = blockIdx.x;
    const int p = b / kp.nObj, o = b % kp.nObj;
    double* sc = ra.scratch + (size_t)b * kRestoreScratch * N2;
    double2* obj = reinterpret_cast<double2*>(sc);
    double* den = sc + 2 * N2;
    double* pt = den + N2;
    double* rr = pt + N2;
    double* tmp = rr + N2;
    int* mask = reinterpret_cast<int*>(tmp + N2);
    __shared__ double noiseVar;
    __shared__ int changed;
    const int first = kp.objFirst[o], cnt = kp.objCount[o];
    const size_t g0 = (size_t)p * kp.I + first;
    // sum_j conj(D_j) S_j and sum_j |S_j|^2 on the support, images in order; conjugate;
    // Array::safeDivide (eps = 0)
    for (int c = threadIdx.x; c < N2; c += THREADS) {
        double2 num = make_double2(0, 0);
        double d = 0;
        if (kp.otfMask[c]) {
            for (int j = 0; j < cnt; ++j) {
                const cx<T> Dv = kp.D[(g0 + j) * N2 + c];
                const cx<T> S = kp.S[(g0 + j) * N2 + c];
                const double dr = Dv.x, di = Dv.y, sr = S.x, si = S.y;
                d += sr * sr + si * si;
                num.x += dr * sr + di * si;   // conj(D) S
                num.y += dr * si - di * sr;
            }
        }
        den[c] = d;
        obj[c] = d != 0.0 ? make_double2(num.x / d, -num.y / d) : make_double2(0, 0);
    }
    if (threadIdx.x == 0) {
        double nv = 0;
        for (int j = 0; j < cnt; ++j) nv += kp.statNoise[g0 + j] * kp.statNoise[g0 + j];
        noiseVar = cnt ? nv / cnt : 0.0;
    }
    __syncthreads();
    if (!ra.noFilter && cnt) {
        const double noiseFactor = noiseVar * N * N;
        for (int c = threadIdx.x; c < N2; c += THREADS)
            tmp[c] = (obj[c].x * obj[c].x + obj[c].y * obj[c].y) * den[c];
        __syncthreads();
        restore_smooth<N, THREADS>(tmp, pt, 1, 1);
        for (int c = threadIdx.x; c < N2; c += THREADS) pt[c] = noiseFactor / pt[c];
        __syncthreads();
        // rr(y, x) = max(1 - (pt(-y, -x) + pt(y, x)) / 2, 0), clipped to {0} u [0.2, 1]
        for (int c = threadIdx.x; c < N2; c += THREADS) {
            const int y = c / N, x = c % N;
            double v = 1.0 - 0.5 * (pt[((N - y) % N) * N + (N - x) % N] + pt[c]);
            v = v > 0.0 ? v : 0.0;
            if (v < 0.2) v = 0.0;
            if (v > 1.0) v = 1.0;
            if (c == (N / 2) * N + N / 2) v = 1.0;     // DC gain = 1
            rr[c] = v;
            mask[c] = (c == (N / 2) * N + N / 2) ? 1 : 0;
        }
        __syncthreads();
        // connectedRegion: the 4-connected region of rr > 0 around the centre, grown until it
        // stops changing (at most N * N sweeps)
        for (int it = 0; it < N2; ++it) {
            if (threadIdx.x == 0) changed = 0;
            __syncthreads();
            int any = 0;
            for (int c = threadIdx.x; c < N2; c += THREADS) {
                if (mask[c] || !(rr[c] > 0.0)) continue;
                const int y = c / N, x = c % N;
                if ((y > 0 && mask[c - N]) || (y < N - 1 && mask[c + N]) || (x > 0 && mask[c - 1]) ||
                    (x < N - 1 && mask[c + 1])) {
                    mask[c] = 1;
                    any = 1;
                }
            }
            if (any) changed = 1;
            __syncthreads();
            if (!changed) break;
        }
        for (int c = threadIdx.x; c < N2; c += THREADS) rr[c] = mask[c] ? rr[c] : 0.0;
        __syncthreads();
        restore_smooth<N, THREADS>(rr, tmp, 4, 4);
        const double fc = 0.9 * ra.fc[o];
        const double fc2 = fc * fc;
        for (int c = threadIdx.x; c < N2; c += THREADS) {
            const int y = c / N, x = c % N;
            const double r2 = (double)(y - N / 2) * (y - N / 2) + (double)(x - N / 2) * (x - N / 2);
            obj[c] = r2 > fc2 ? make_double2(0, 0) : make_double2(obj[c].x * tmp[c], obj[c].y * tmp[c]);
        }
        __syncthreads();
    }
    // ift: un-centre, backward transform, real part / N^2.  The rows and then the columns
    // are transformed in bands of kRestoreBand lines through shared memory (an N x N FP64
    // tile does not fit for N = 128); the row results go to W (the den and pt arrays).
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int B = kRestoreBand;
    cx<double>* s = reinterpret_cast<cx<double>*>(smem_raw);     // [B][LDS]
    cx<double>* tw = s + B * LDS;
    cx<double>* W = reinterpret_cast<cx<double>*>(den);
    for (int k = threadIdx.x; k < N; k += THREADS) {
        double sn, cs;
        sincospi(2.0 * k / N, &sn, &cs);
        tw[k] = mkc<double>(cs, -sn);
    }
    for (int r0 = 0; r0 < N; r0 += B) {
        __syncthreads();
        for (int i = threadIdx.x; i < B * N; i += THREADS) {
            const int y = r0 + i / N, x = i % N;
            const double2 v = obj[((y + N / 2) % N) * N + (x + N / 2) % N];
            s[(i / N) * LDS + x] = mkc<double>(v.x, v.y);
        }
        __syncthreads();
        fft_lines<double, N, +1, B, true, THREADS>(s, 0, tw, threadIdx.x);
        for (int i = threadIdx.x; i < B * N; i += THREADS) W[(r0 + i / N) * N + i % N] = s[(i / N) * LDS + i % N];
    }
    const int ps = kp.ps, off = (N - ps) / 2;
    float* out = ra.out + ((size_t)p * kp.nObj + o) * ps * ps;
    for (int c0 = 0; c0 < N; c0 += B) {
        __syncthreads();
        for (int i = threadIdx.x; i < B * N; i += THREADS) {
            const int col = c0 + i % B, y = i / B;
            s[(i % B) * LDS + y] = W[y * N + col];
        }
        __syncthreads();
        fft_lines<double, N, +1, B, true, THREADS>(s, 0, tw, threadIdx.x);
        for (int i = threadIdx.x; i < B * N; i += THREADS) {
            const int x = c0 + i / N, y = i % N;
            if (x >= off && x < off + ps && y >= off && y < off + ps)
                out[(y - off) * ps + (x - off)] = (float)(s[(i / N) * LDS + y].x / (double)N2);
        }
    }
}

}  // namespace rdxg
