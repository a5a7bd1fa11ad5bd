// Definitions of Launcher<T, N>; included once per OTF size by rdxg_inst_<N>.cu.
#pragma once

#include <type_traits>

#include "rdxg_launch.h"

namespace rdxg {

// FP32 handles have a second block size of k_forward and k_adjoint for the planner; the FP64
// form (the plain baseline) keeps one.
template <typename T> struct HasAlt { static constexpr bool value = std::is_same<T, float>::value; };

// after the work tile and twiddles: the larger of the alpha staging, the adjoint's projection
// weights [n2] and mode sums [M] (8 bytes each), a reduction buffer
template <typename T, int N>
static size_t extra_smem(int M) {
    size_t a = (size_t)M * sizeof(T);
    size_t b = (size_t)(N / 2) * (N / 2) * sizeof(T) + (size_t)M * 8;
    size_t c = 33 * sizeof(double);
    size_t m = a > b ? a : b;
    return (m > c ? m : c) + 16;
}

template <typename T, int N>
static size_t smem_pp(int M) {
    return (size_t)(PingPong<T, N>::value ? Tile<N>::ELEMS : 0) * sizeof(cx<T>) + Launcher<T, N>::smem_base() +
           extra_smem<T, N>(M);
}

// shared memory of the recomputing adjoint: tile [| X tile] | twiddles | PF | projection
// weights | alpha, then the mode sums (8 bytes per mode) in its place
template <typename T, int N>
static size_t adjoint_rc_smem(int M) {
    constexpr size_t n2 = (size_t)(N / 2) * (N / 2);
    constexpr size_t tiles = PingPong<T, N>::value ? 2 : 1;
    return (size_t)(tiles * Tile<N>::ELEMS + N + n2) * sizeof(cx<T>) + n2 * sizeof(T) + (size_t)M * 8 + 16;
}
// ... of the recomputing finite-difference gradient: k_fd's | PF | alpha
template <typename T, int N>
static size_t fd_rc_smem(int M) {
    constexpr size_t n2 = (size_t)(N / 2) * (N / 2);
    return ((fd_base_smem<T, N>() + 15) & ~(size_t)15) + n2 * sizeof(cx<T>) + (size_t)M * sizeof(T) + 16;
}

template <typename T, int N>
cudaError_t Launcher<T, N>::setup(int M) {
    const int sm = (int)smem_pp<T, N>(M);
    cudaError_t e;
    if ((e = raise_smem_limit(k_prep<T, N, THREADS>, sm))) return e;
    if ((e = raise_smem_limit(k_forward<T, N, THREADS>, sm))) return e;
    if ((e = raise_smem_limit(adjoint_kernel<T, N, THREADS>(), sm))) return e;
    if ((e = raise_smem_limit(k_fd<T, N, THREADS>, sm))) return e;
    const size_t arc = adjoint_rc_smem<T, N>(M), frc = fd_rc_smem<T, N>(M);
    if (arc <= kMaxSmem && (e = raise_smem_limit(k_adjoint_rc<T, N, THREADS, false>, arc))) return e;
    if (frc <= kMaxSmem && (e = raise_smem_limit(k_fd_rc<T, N, THREADS>, frc))) return e;
    if constexpr (HasAlt<T>::value) {
        constexpr int ALT = ThreadsAlt<N>::value;
        if ((e = raise_smem_limit(k_forward<T, N, ALT>, sm))) return e;
        if ((e = raise_smem_limit(adjoint_kernel<T, N, ALT>(), sm))) return e;
        if (arc <= kMaxSmem && (e = raise_smem_limit(k_adjoint_rc<T, N, ALT, false>, arc))) return e;
        if constexpr (PlanAlt<N>::exists) {
            using PA = PlanAlt<N>;
            if ((e = raise_smem_limit(k_forward<T, N, THREADS, PA>, sm))) return e;
            if ((e = raise_smem_limit(adjoint_kernel<T, N, THREADS, PA>(), sm))) return e;
            if ((e = raise_smem_limit(k_forward<T, N, ALT, PA>, sm))) return e;
            if ((e = raise_smem_limit(adjoint_kernel<T, N, ALT, PA>(), sm))) return e;
        }
    }
    if constexpr (PingPong<T, N>::value) {
        // the fused path recomputes S too
        if (arc <= kMaxSmem && (e = raise_smem_limit(k_adjoint_rc<T, N, THREADS, true>, arc))) return e;
        if (arc <= kMaxSmem && (e = raise_smem_limit(k_adjoint_rc<T, N, ThreadsAlt<N>::value, true>, arc))) return e;
    }
    return cudaSuccess;
}

template <typename T, int N>
int Launcher<T, N>::recompute_occupancy(int M) {
    if (adjoint_rc_smem<T, N>(M) > kMaxSmem || fd_rc_smem<T, N>(M) > kMaxSmem) return 0;
    int a = 0, f = 0;
    // the larger block size of the adjoint's two shapes has the same or a lower occupancy
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, k_adjoint_rc<T, N, THREADS, PingPong<T, N>::value>, THREADS,
                                                  adjoint_rc_smem<T, N>(M));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, k_fd_rc<T, N, THREADS>, THREADS, fd_rc_smem<T, N>(M));
    const int occ = a > f ? a : f;
    return occ < 1 ? 1 : (occ > 32 ? 32 : occ);
}

template <typename T, int N>
void Launcher<T, N>::prep(const KParams<T>& kp, int full, int nImg, cudaStream_t st) {
    const size_t sm = smem_base() + extra_smem<T, N>(kp.M);
    k_prep<T, N, THREADS><<<nImg, THREADS, sm, st>>>(kp, full);
}

template <typename T, int N>
void Launcher<T, N>::forward(const KParams<T>& kp, int nImg, cudaStream_t st) {
    const size_t sm = smem_base() + extra_smem<T, N>(kp.M);
    if constexpr (HasAlt<T>::value) {
        // the planner's variant: bit 0 the alternative block size, bit 1 the alternative radix plan
        constexpr int ALT = ThreadsAlt<N>::value;
        if constexpr (PlanAlt<N>::exists) {
            using PA = PlanAlt<N>;
            if (kp.shapeFwd == 2) { k_forward<T, N, THREADS, PA><<<nImg, THREADS, sm, st>>>(kp); return; }
            if (kp.shapeFwd == 3) { k_forward<T, N, ALT, PA><<<nImg, ALT, sm, st>>>(kp); return; }
        }
        if (kp.shapeFwd == 1) {
            k_forward<T, N, ALT><<<nImg, ALT, sm, st>>>(kp);
            return;
        }
    }
    k_forward<T, N, THREADS><<<nImg, THREADS, sm, st>>>(kp);
}

template <typename T, int N>
void Launcher<T, N>::adjoint(const KParams<T>& kp, int grid, int kind, cudaStream_t st) {
    (void)grid;
    if (kp.recompute) {
        // one image per block; S recomputed where it is not kept (the fused path)
        const size_t sm = adjoint_rc_smem<T, N>(kp.M);
        const int g = kp.P * kp.I;
        const bool alt = HasAlt<T>::value && (kp.shapeAdj & 1);
        if constexpr (PingPong<T, N>::value) {
            if (!kp.S) {
                if (alt) k_adjoint_rc<T, N, ThreadsAlt<N>::value, true><<<g, ThreadsAlt<N>::value, sm, st>>>(kp, kind);
                else k_adjoint_rc<T, N, THREADS, true><<<g, THREADS, sm, st>>>(kp, kind);
                return;
            }
        }
        if constexpr (HasAlt<T>::value) {
            if (alt) {
                k_adjoint_rc<T, N, ThreadsAlt<N>::value, false><<<g, ThreadsAlt<N>::value, sm, st>>>(kp, kind);
                return;
            }
        }
        k_adjoint_rc<T, N, THREADS, false><<<g, THREADS, sm, st>>>(kp, kind);
        return;
    }
    const size_t sm = smem_base() + extra_smem<T, N>(kp.M);
    grid = kp.P * kp.I;
    if constexpr (HasAlt<T>::value) {
        constexpr int ALT = ThreadsAlt<N>::value;
        if constexpr (PlanAlt<N>::exists) {
            using PA = PlanAlt<N>;
            if (kp.shapeAdj == 2) { adjoint_kernel<T, N, THREADS, PA>()<<<grid, THREADS, sm, st>>>(kp, kind); return; }
            if (kp.shapeAdj == 3) { adjoint_kernel<T, N, ALT, PA>()<<<grid, ALT, sm, st>>>(kp, kind); return; }
        }
        if (kp.shapeAdj == 1) {
            adjoint_kernel<T, N, ALT>()<<<grid, ALT, sm, st>>>(kp, kind);
            return;
        }
    }
    adjoint_kernel<T, N, THREADS>()<<<grid, THREADS, sm, st>>>(kp, kind);
}

template <typename T, int N>
void Launcher<T, N>::fd(const KParams<T>& kp, int grid, int M, cudaStream_t st) {
    if (kp.recompute) {
        const int g = PingPong<T, N>::value ? kp.scrBlocks : kp.P * kp.I * M;
        k_fd_rc<T, N, THREADS><<<g, THREADS, fd_rc_smem<T, N>(kp.M), st>>>(kp);
        return;
    }
    const size_t sm = smem_pp<T, N>(kp.M);
    if (!PingPong<T, N>::value) grid = kp.P * kp.I * M;
    if (GlobalTile<T, N>::value) grid = grid < kp.gtileBlocks ? grid : kp.gtileBlocks;   // one tile per block
    k_fd<T, N, THREADS><<<grid, THREADS, sm, st>>>(kp);
}

template <typename T, int N>
cudaError_t Launcher<T, N>::restore(const KParams<T>& kp, const RestoreArgs& ra, int nBlocks, cudaStream_t st) {
    const int sm = (int)((size_t)(kRestoreBand * Tile<N>::LDS + N) * sizeof(cx<double>));
    k_restore<T, N, THREADS><<<nBlocks, THREADS, sm, st>>>(kp, ra);
    return cudaGetLastError();   // the launch only (no device synchronisation)
}

template <typename T, int N>
cudaError_t Launcher<T, N>::restore_outputs(const KParams<T>& kp, const RestoreOutArgs& oa, int grid,
                                            cudaStream_t st) {
    const int sm = (int)((size_t)(kRestoreBand * Tile<N>::LDS + N) * sizeof(cx<double>));
    const int nPo = kp.P * kp.nObj, nImg = kp.P * kp.I;
    k_restore_objft<T, N, THREADS><<<grid < nPo ? grid : nPo, THREADS, sm, st>>>(kp, oa);
    if (oa.flags & (kRestorePsf | kRestoreCobj | kRestoreResidual))
        k_restore_images<T, N, THREADS><<<grid < nImg ? grid : nImg, THREADS, sm, st>>>(kp, oa);
    return cudaGetLastError();
}

template <typename T, int N>
size_t EvalLauncher<T, N>::smem(int M, int nH) {
    (void)M;
    // two tiles | twiddles | reference object | pupil amplitude | phases of the image | tile
    // positions (16-bit); the accumulators live in registers
    return (size_t)(2 * Tile<N>::ELEMS + N + nH) * sizeof(cx<T>) + (size_t)2 * (N / 2) * (N / 2) * sizeof(T) +
           (size_t)nH * sizeof(uint16_t) + 16;
}

#define RDXG_NPT_SWITCH(npt, CALL) \
    do {                             \
        (void)(npt);                 \
        CALL(1);                     \
    } while (0)

template <typename T, int N>
cudaError_t EvalLauncher<T, N>::setup(int M, int npt, int nH) {
    cudaError_t e = cudaSuccess;
    const int sm = (int)smem(M, nH);
#define RDXG_SET(NPT) e = raise_smem_limit(k_eval<T, N, kEvalThreads, NPT>, sm)
    RDXG_NPT_SWITCH(npt, RDXG_SET);
#undef RDXG_SET
#define RDXG_SET(NPT) e = raise_smem_limit(k_eval<T, N, kEvalThreadsAlt, NPT>, sm)
    if (e == cudaSuccess) RDXG_NPT_SWITCH(npt, RDXG_SET);
#undef RDXG_SET
    if constexpr (PlanAlt<N>::exists) {
        if (e == cudaSuccess) e = raise_smem_limit(k_eval<T, N, kEvalThreads, 1, PlanAlt<N>>, sm);
        if (e == cudaSuccess) e = raise_smem_limit(k_eval<T, N, kEvalThreadsAlt, 1, PlanAlt<N>>, sm);
    }
    if (e == cudaSuccess)
        e = raise_smem_limit(k_phase<T, N, kPhasePix, kMaxChunk>, (size_t)M * (kPhasePix + kMaxChunk) * sizeof(T));
    if (e == cudaSuccess && fd_smem(nH) + 1024 <= kMaxSmem)
        e = raise_smem_limit(k_fd_half<T, N, kEvalThreads, false>, fd_smem(nH));
    if (e == cudaSuccess && fd_smem(nH) + 1024 <= kMaxSmem)
        e = raise_smem_limit(k_fd_half<T, N, kEvalThreads, true>, fd_smem(nH));
    return e;
}

template <typename T, int N>
int EvalLauncher<T, N>::occupancy(int M, int npt, int nH) {
    int b = 0;
    const size_t sm = smem(M, nH);
#define RDXG_OCC(NPT) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_eval<T, N, kEvalThreads, NPT>, kEvalThreads, sm)
    RDXG_NPT_SWITCH(npt, RDXG_OCC);
#undef RDXG_OCC
    return b;
}

template <typename T, int N>
void EvalLauncher<T, N>::eval(const EvalParams<T>& e, int npt, int grid, cudaStream_t st) {
    const size_t sm = smem(e.k.M, e.hp.nH);
    // the planner's variant: bit 0 the alternative block size, bit 1 the alternative radix plan
    if constexpr (PlanAlt<N>::exists) {
        if (e.k.shapeEval == 2) { k_eval<T, N, kEvalThreads, 1, PlanAlt<N>><<<grid, kEvalThreads, sm, st>>>(e); return; }
        if (e.k.shapeEval == 3) {
            k_eval<T, N, kEvalThreadsAlt, 1, PlanAlt<N>><<<grid, kEvalThreadsAlt, sm, st>>>(e);
            return;
        }
    }
    if (e.k.shapeEval == 1) {
#define RDXG_LAUNCH(NPT) k_eval<T, N, kEvalThreadsAlt, NPT><<<grid, kEvalThreadsAlt, sm, st>>>(e)
        RDXG_NPT_SWITCH(npt, RDXG_LAUNCH);
#undef RDXG_LAUNCH
        return;
    }
#define RDXG_LAUNCH(NPT) k_eval<T, N, kEvalThreads, NPT><<<grid, kEvalThreads, sm, st>>>(e)
    RDXG_NPT_SWITCH(npt, RDXG_LAUNCH);
#undef RDXG_LAUNCH
}

template <typename T>
static size_t phase_patch_smem(int maxm) {
    return ((size_t)2 * kPhaseMaxImg * maxm + kPhaseMaxCh * kPhaseRegPix) * sizeof(T) + 2 * kPhaseMaxImg * sizeof(int);
}

template <typename T, int N>
int EvalLauncher<T, N>::phase_tiles() {
    return ((N / 2) * (N / 2) + kPhaseRegPix - 1) / kPhaseRegPix;
}

template <typename T, int N>
void EvalLauncher<T, N>::phase(const EvalParams<T>& e, int grid, cudaStream_t st) {
    if constexpr (std::is_same<T, float>::value) {
        if (e.Zt && e.tc.valid) {
            PhaseTcArgs a;
            a.Zt = e.Zt; a.alphaEff = e.k.alphaEff; a.phiFixed = e.k.phiFixed; a.imgCh = e.k.pImgCh;
            a.evalP = e.L.evalP; a.nEvalP = e.L.nEvalP; a.phi = e.phi; a.status = e.tcStatus;
            a.I = e.k.I; a.M = e.k.M; a.n2 = (N / 2) * (N / 2); a.nCh = e.nCh;
            a.G = e.tc.G; a.NT = e.tc.NT; a.KP = e.tc.KP; a.parts = e.tc.parts;
            launch_phase_tc(a, e.tc, st);
            return;
        }
    }
    if (e.k.M <= kPhaseRegModes && e.nCh <= kPhaseMaxCh && e.k.I <= kPhaseMaxImg) {
        // grid: a multiple of the pixel tiles
        const int nPix = phase_tiles();
        const int g = (grid / nPix > 0 ? grid / nPix : 1) * nPix;
#define RDXG_PHASE_PATCH(MM)                                                                     \
    k_phase_patch<T, N, kPhaseRegPix, MM, kPhaseMaxImg, kPhaseMaxCh>                              \
        <<<g, kPhaseRegPix, phase_patch_smem<T>(MM), st>>>(e)
        switch ((e.k.M + 7) / 8) {
            case 0: case 1: RDXG_PHASE_PATCH(8); break;
            case 2: RDXG_PHASE_PATCH(16); break;
            case 3: RDXG_PHASE_PATCH(24); break;
            case 4: RDXG_PHASE_PATCH(32); break;
            case 5: RDXG_PHASE_PATCH(40); break;
            case 6: RDXG_PHASE_PATCH(48); break;
            case 7: RDXG_PHASE_PATCH(56); break;
            default: RDXG_PHASE_PATCH(64); break;
        }
#undef RDXG_PHASE_PATCH
        return;
    }
    const size_t sm = (size_t)e.k.M * (kPhasePix + kMaxChunk) * sizeof(T);
    k_phase<T, N, kPhasePix, kMaxChunk><<<grid, kPhasePix, sm, st>>>(e);
}

template <typename T, int N>
size_t EvalLauncher<T, N>::fd_smem(int nH) {
    return (size_t)(2 * Tile<N>::ELEMS + N + (N / 2) * (N / 2) + 2 * nH) * sizeof(cx<T>) +
           (size_t)2 * nH * sizeof(T) + (size_t)nH * sizeof(unsigned short) + 16;
}

template <typename T, int N>
void EvalLauncher<T, N>::fd_half(const EvalParams<T>& e, int grid, cudaStream_t st) {
    // one block size only: its per-thread partial sums of the metric change depend on it
    // recomputed transforms: X of the block's image in its scratch slot (slot = block)
    if (e.k.recompute) k_fd_half<T, N, kEvalThreads, true><<<grid, kEvalThreads, fd_smem(e.hp.nH), st>>>(e);
    else k_fd_half<T, N, kEvalThreads, false><<<grid, kEvalThreads, fd_smem(e.hp.nH), st>>>(e);
}

template <typename T, int N>
void EvalLauncher<T, N>::reduce(const EvalParams<T>& e, int grid, cudaStream_t st) {
    k_reduce<T, N, kReduceThreads><<<grid, kReduceThreads, 0, st>>>(e);
}

}  // namespace rdxg
