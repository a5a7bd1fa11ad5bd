// C ABI of the batched MOMFBD solver core (include/rdxg.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <chrono>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/rdxg.h"
#include "rdxg_launch.h"

using namespace rdxg;

namespace {

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

}  // namespace

struct rdxg_solver {
    rdxg_geometry geo{};
    int N = 0, n = 0, ps = 0, cs = 0, margin = 0, M = 0, I = 0, nObj = 0, C = 0, nPar = 0, nFree = 0;
    int Pmax = 0, P = 0, nTiles = 0;
    bool fp64 = false;
    cudaStream_t own = nullptr, stream = nullptr;
    std::string err;
    std::vector<void*> allocs;
    // host copies
    std::vector<int32_t> imgObj, imgCh, objFirst, objCount;
    std::vector<double> objWeight, gradStep;
    double J[2][2] = {{0, 0}, {0, 0}}, Jinv[2][2] = {{0, 0}, {0, 0}};
    bool haveJ = false;
    double area = 0;
    // device static
    void *dZ = nullptr, *dA = nullptr, *dPhi = nullptr, *dOtfNorm = nullptr, *dTw = nullptr;
    uint8_t* dMask = nullptr;
    int32_t *dImgObj = nullptr, *dImgCh = nullptr, *dObjFirst = nullptr, *dObjCount = nullptr;
    const int32_t *dObjFirstC = nullptr, *dObjCountC = nullptr;
    double *dObjW = nullptr, *dGradStep = nullptr, *dWin = nullptr, *dNWin = nullptr;
    double* dGradScale = nullptr;     // [2][nObj][C] the adjoint's factors (Vogel, exact)
    int32_t *dRowPtr = nullptr, *dRowCol = nullptr, *dColPtr = nullptr, *dColRow = nullptr;
    double *dRowVal = nullptr, *dColVal = nullptr;
    float* dRowVal32 = nullptr;   // FP32 copy of the row values (metric requests of the FP32 path)
    // device per patch
    float* dCut = nullptr;
    const float* dCutExt = nullptr;   // caller-owned device cutouts
    int32_t* dShift = nullptr;
    double *dMean = nullptr, *dStd = nullptr, *dNoise = nullptr, *dRg = nullptr;
    void *dAlphaEff = nullptr, *dD = nullptr, *dS = nullptr, *dX = nullptr, *dPF = nullptr, *dO = nullptr, *dQt = nullptr;
    double *dGamma = nullptr, *dPartial = nullptr, *dGalpha = nullptr;
    int32_t *dReq = nullptr, *dGm = nullptr, *dMc = nullptr;
    uint8_t* dReinit = nullptr;
    double *dCurTilt = nullptr, *dResAlpha = nullptr;
    // solver state
    CgState* dStates = nullptr;
    double *dVec = nullptr, *dMetrics = nullptr, *dAlpha = nullptr, *dAlphaOff = nullptr;
    float* dAlphaOffF = nullptr;      // [P][nPar] alpha offsets rounded to float
    int32_t* dActive = nullptr;
    int32_t* hActive = nullptr;   // pinned
    int maxMetrics = 0;
    bool loaded = false, dirty = false;
    std::vector<double> hResAlpha, hFixedGamma;
    bool haveFixedGamma = false;
    int64_t launches = 0;
    rdxg_solve_params lastParams{};
    // fused evaluation path (FP32, N <= 88)
    bool fused = false;
    cudaStream_t side = nullptr;     // capture stream of the graph's conditional bodies
    unsigned long long* dLaunchCount = nullptr;   // kernel launches of a graph-run solve
    // device loop of a solve graph (on the first handle of a solve): the handles' active
    // counters, the rounds run and the overrun flag
    int32_t** dActiveList = nullptr;
    int activeListCap = 0;
    long long* dRounds = nullptr;
    int32_t* dOverrun = nullptr;
    double* dRestore = nullptr;      // restoration scratch (allocated on first use)
    double* dFc = nullptr;           // [nObj] frequency cutoffs of the restoration
    float* dRestoreOut = nullptr;    // [P][nObj][ps][ps] restored objects
    // optional restoration outputs (allocated on first use)
    float *dObjFull = nullptr, *dPsf = nullptr, *dCobj = nullptr, *dRes = nullptr;
    double *dFo = nullptr, *dOutPool = nullptr;
    bool fusedFd = false;     // half-plane finite-difference gradient (fits in shared memory)
    int npt = 0, chunk = 6, chunksPerPatch = 0, nH = 0, evalGrid = 0, reduceGrid = 0, numSMs = 0;
    std::vector<int32_t> objChunk0, hIdx, hPos;
    int nTilesH = 0;
    int32_t *dHPos = nullptr;
    int32_t *dHIdx = nullptr, *dObjChunk0 = nullptr, *dCounters = nullptr, *dAux = nullptr;
    void *dDh = nullptr, *dOh = nullptr, *dPart = nullptr, *dPhiImg = nullptr;
    int phaseGrid = 0;
    double* dObjMetric = nullptr;
    EvalItem* dEval = nullptr;
    PoItem* dPoList = nullptr;
    int32_t *dGradP = nullptr, *dFdP = nullptr, *dEvalP = nullptr;
    int adjGrid = 0, fdGrid = 0;
    // mode expansion of the fused path: 0 CUDA cores (FP32), 2 tensor cores 3xBF16, 3 6xBF16
    int phaseParts = 3;
    PhaseTcPlan tcPlan{};
    __nv_bfloat16* dZt = nullptr;    // split modes (room for three parts)
    int32_t* dTcStatus = nullptr;
    // launch shapes (0 default block size, 1 the alternative) and how they are chosen:
    // tune 1 = measured on the first solve (or taken from the planner's table), 0 = pinned
    int shapeEval = 0, shapeFwd = 0, shapeAdj = 0;
    int tune = 1;
    bool tuned = false;
    // FIT_PLANE: the fitted plane of every (patch, object), slopes along y and x
    bool fitPlane = false;
    double* dPlane = nullptr;
    // warm start: the initial coefficients of the loaded patches [P][I][M] (loadInit)
    bool haveInit = false;
    bool initRecut = true;           // false: rdxg_set_start_alpha (the images stay as loaded)
    double* dInitAlpha = nullptr;
    // REG_ALPHA: per-parameter weights [I][M] of 0.5 sum alpha^2 w (Solver::regAlphaWeights)
    std::vector<double> hRegW;
    double* dRegW = nullptr;
    // rdxg_metric_noalloc: address of the library's static scratch in this handle's context,
    // looked up when the handle is created (fused handles only)
    void* dNoAlloc = nullptr;
    // recomputed transforms: X and PF (and on the fused path S) are not kept per image; the
    // gradient kernels form them again with one scratch slot of N^2 per resident block
    bool recompute = false;
    void* dXscr = nullptr;           // [nsmid * slotsPerSM][N*N] scratch tiles
    int scrBlocks = 0;               // blocks of the persistent recomputing kernels
    int nsmid = 0, slotsPerSM = 0;   // SM identifiers (%nsmid), slots per SM (occupancy)
    unsigned* dSlotMask = nullptr;   // [nsmid] slots in use
    int32_t* dRcStatus = nullptr;    // a block of a recomputing kernel found no free slot
    size_t allocBytes = 0;           // device bytes the handle holds
    // global work tiles of the transform kernels where a tile does not fit shared memory
    void* dGtile = nullptr;
    int gtileBlocks = 0;
    // patch shapes: shape 0 is the handle's own geometry (every image and mode, the static
    // null space); rdxg_set_patch_shapes adds those of a ragged batch and gives each patch one.
    // On the device: every patch's geometry and image/object tables, every shape's maps.
    struct Shape {
        int frames = -1, M = 0, nFree = 0, nImg = 0, chunks = 0;
        std::vector<int32_t> imgObj, imgCh, objFirst, objCount, objChunk0;   // [I] / [nObj]
        std::vector<int32_t> rowPtr, rowCol, colPtr, colRow;                // rows: slot * M + mode
        std::vector<double> rowVal, colVal;
    };
    std::vector<Shape> shapes;
    std::vector<int32_t> patchShape;   // [Pmax]
    bool ragged = false;
    int raggedPatches = 0;             // patches the shapes were given for
    PatchGeo* dPGeo = nullptr;
    int32_t *dPImgObj = nullptr, *dPImgCh = nullptr, *dPObjFirst = nullptr, *dPObjCount = nullptr,
            *dPObjChunk0 = nullptr;
    size_t mapRowEntries = 0, mapColEntries = 0, mapNnz = 0;   // sizes of the device maps
    int32_t mapMaxNnz = 0;            // the largest row-map entry count of a patch shape
    int32_t cgStage = 0, cgStageMap = 0;   // the solver kernel's staged form (set per solve)
    int32_t cgForm = 0;               // pinned solver kernel form (0: staged when it fits)
};

namespace {

#define CK(h, call)                                                                            \
    do {                                                                                       \
        cudaError_t _e = (call);                                                               \
        if (_e != cudaSuccess) {                                                               \
            (h)->err = std::string(#call) + ": " + cudaGetErrorString(_e);                     \
            return RDXG_ERR_CUDA;                                                              \
        }                                                                                      \
    } while (0)

#define CKL(h)                                                                                 \
    do {                                                                                       \
        cudaError_t _e = cudaGetLastError();                                                   \
        if (_e != cudaSuccess) {                                                               \
            (h)->err = std::string("kernel launch: ") + cudaGetErrorString(_e);               \
            return RDXG_ERR_CUDA;                                                              \
        }                                                                                      \
    } while (0)

int dalloc(rdxg_solver* h, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        h->err = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return RDXG_ERR_NOMEM;
    }
    h->allocs.push_back(*p);
    h->allocBytes += bytes;
    return RDXG_OK;
}

// frees one allocation of the handle (bytes: its size, for the tally) and clears the pointer
template <typename P>
void dfree(rdxg_solver* h, P** p, size_t bytes) {
    if (!*p) return;
    for (auto it = h->allocs.begin(); it != h->allocs.end(); ++it)
        if (*it == (void*)*p) {
            cudaFree(*it);
            h->allocs.erase(it);
            h->allocBytes -= bytes ? bytes : 16;
            break;
        }
    *p = nullptr;
}

template <typename P>
int dalloc_t(rdxg_solver* h, P** p, size_t count) {
    void* v = nullptr;
    int r = dalloc(h, &v, count * sizeof(P));
    *p = static_cast<P*>(v);
    return r;
}

template <typename T>
int upload(rdxg_solver* h, void** dst, const std::vector<T>& v) {
    int r = dalloc(h, dst, v.size() * sizeof(T));
    if (r) return r;
    CK(h, cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return RDXG_OK;
}

bool supported_N(int N) { return N == 32 || N == 64 || N == 88 || N == 128; }

// dispatch on (precision, N)
template <typename F>
void with_size(int N, bool fp64, F&& f) {
#define RDXG_CASE(NN)                                                  \
    case NN:                                                           \
        if (fp64) f(Launcher<double, NN>{}, double{}); else f(Launcher<float, NN>{}, float{}); \
        break;
    switch (N) {
        RDXG_CASE(32)
        RDXG_CASE(64)
        RDXG_CASE(88)
        RDXG_CASE(128)
        default: break;
    }
#undef RDXG_CASE
}

template <typename F>
void with_eval(int N, F&& f) {
    switch (N) {
        case 32: f(EvalLauncher<float, 32>{}); break;
        case 64: f(EvalLauncher<float, 64>{}); break;
        case 88: f(EvalLauncher<float, 88>{}); break;
        default: break;
    }
}

template <typename T>
KParams<T> make_kparams(rdxg_solver* h) {
    KParams<T> k{};
    k.P = h->P; k.I = h->I; k.M = h->M; k.nObj = h->nObj; k.N = h->N; k.n = h->n;
    k.ps = h->ps; k.cs = h->cs; k.margin = h->margin; k.nTiles = h->nTiles;
    k.Z = (const T*)h->dZ; k.A = (const T*)h->dA; k.phiFixed = (const T*)h->dPhi;
    k.otfNorm = (const T*)h->dOtfNorm; k.otfMask = h->dMask;
    k.pgeo = h->dPGeo; k.pImgObj = h->dPImgObj; k.pImgCh = h->dPImgCh;
    k.pObjFirst = h->dPObjFirst; k.pObjCount = h->dPObjCount;
    k.objWeight = h->dObjW; k.objGradStep = h->dGradStep; k.window = h->dWin; k.noiseWindow = h->dNWin;
    k.tw = (const cx<T>*)h->dTw; k.area = h->area; k.tiltX = h->geo.tilt_x; k.tiltY = h->geo.tilt_y;
    k.gradScale = h->dGradScale; k.nCh = h->C;
    k.cutouts = h->dCutExt ? h->dCutExt : h->dCut;
    k.shift = h->dShift; k.statMean = h->dMean; k.statStd = h->dStd; k.statNoise = h->dNoise; k.rg = h->dRg;
    k.alphaEff = (const T*)h->dAlphaEff;
    k.D = (cx<T>*)h->dD; k.S = (cx<T>*)h->dS; k.X = (cx<T>*)h->dX; k.PF = (cx<T>*)h->dPF;
    k.O = (cx<T>*)h->dO; k.Qt = (T*)h->dQt;
    k.gamma = h->dGamma; k.partial = h->dPartial; k.galpha = h->dGalpha;
    k.req = h->dReq; k.gmethod = h->dGm; k.modeCount = h->dMc; k.reinit = h->dReinit;
    k.Dh = (cx<T>*)h->dDh; k.hIdx = h->dHIdx; k.nH = h->nH;
    k.gradP = h->dGradP; k.nGradP = h->dCounters + 2; k.fdP = h->dFdP; k.nFdP = h->dCounters + 3;
    k.shapeEval = h->shapeEval; k.shapeFwd = h->shapeFwd; k.shapeAdj = h->shapeAdj;
    k.plane = h->fitPlane ? h->dPlane : nullptr;
    k.recompute = h->recompute ? 1 : 0;
    k.phiImg = (h->fused || h->tcPlan.valid) ? (const T*)h->dPhiImg : nullptr;
    k.Xscr = (cx<T>*)h->dXscr;
    k.scrBlocks = h->scrBlocks;
    k.slotMask = h->dSlotMask;
    k.slotsPerSM = h->slotsPerSM;
    k.rcStatus = h->dRcStatus;
    k.gtile = (cx<T>*)h->dGtile;
    k.gtileBlocks = h->gtileBlocks;
    return k;
}

Lists make_lists(rdxg_solver* h) {
    Lists L{};
    L.eval = h->dEval; L.po = h->dPoList;
    L.counters = h->dCounters;
    L.nEval = h->dCounters + 0; L.nPo = h->dCounters + 1;
    L.gradP = h->dGradP; L.nGradP = h->dCounters + 2;
    L.fdP = h->dFdP; L.nFdP = h->dCounters + 3;
    L.evalP = h->dEvalP; L.nEvalP = h->dCounters + 4;
    return L;
}

template <typename T>
EvalParams<T> make_evalparams(rdxg_solver* h) {
    EvalParams<T> e{};
    e.k = make_kparams<T>(h);
    e.hp.nH = h->nH; e.hp.idx = h->dHIdx; e.hp.chunkSize = h->chunk;
    e.hp.chunksPerPatch = h->chunksPerPatch; e.hp.objChunk0 = h->dPObjChunk0;
    e.Dh = (const cx<T>*)h->dDh; e.Oh = (cx<T>*)h->dOh; e.part = (Acc4<T>*)h->dPart;
    e.objMetric = h->dObjMetric; e.L = make_lists(h);
    e.hPos = h->dHPos; e.nTilesH = h->nTilesH; e.phi = (T*)h->dPhiImg;
    e.nCh = h->C;
    e.Zt = h->tcPlan.valid ? h->dZt : nullptr;
    e.tcStatus = h->dTcStatus;
    e.tc = h->tcPlan;
    return e;
}

// Chooses the mode expansion of the fused path and splits the modes for the tensor cores.
int setup_phase_tc(rdxg_solver* h, int parts) {
    h->phaseParts = parts;
    h->tcPlan = PhaseTcPlan{};
    if (parts == 0) return RDXG_OK;
    const int n2 = h->n * h->n;
    if (!h->dZt) {
        const PhaseTcPlan p3 = phase_tc_plan(h->I, h->M, n2, h->C, 3, h->numSMs);
        const PhaseTcPlan p2 = phase_tc_plan(h->I, h->M, n2, h->C, 2, h->numSMs);
        const size_t elems = p3.valid ? p3.zElems : p2.zElems;
        if (!p2.valid) return RDXG_OK;   // shape the tensor-core kernel does not take: CUDA cores
        int r;
        if ((r = dalloc(h, (void**)&h->dZt, elems * sizeof(__nv_bfloat16))) || (r = dalloc_t(h, &h->dTcStatus, 1)))
            return r;
        CK(h, cudaMemsetAsync(h->dTcStatus, 0, sizeof(int32_t), h->stream));
    }
    const PhaseTcPlan p = phase_tc_plan(h->I, h->M, n2, h->C, parts, h->numSMs);
    cudaGetLastError();
    if (!p.valid) return RDXG_OK;
    launch_tc_pack_modes((const float*)h->dZ, (const float*)h->dPhi, h->M, h->C, n2, p, h->dZt, h->stream);
    CKL(h);
    CK(h, cudaStreamSynchronize(h->stream));
    h->tcPlan = p;
    if (getenv("RDXG_VERBOSE"))
        fprintf(stderr, "tensor-core mode expansion: parts %d, K %d, images per tile %d (%d patches), smem %zu, "
                "occupancy %d, grid %d\n", p.parts, p.KP, p.NT, p.G, p.smem, p.occ, p.grid);
    return RDXG_OK;
}

// Reports (once) a wait of the tensor-core mode expansion that gave up, or a block of the
// recomputing kernels that found no scratch slot.
int tc_check(rdxg_solver* h) {
    if (h->dRcStatus) {
        int32_t st = 0;
        CK(h, cudaMemcpyAsync(&st, h->dRcStatus, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
        if (st) {
            CK(h, cudaMemsetAsync(h->dRcStatus, 0, sizeof(int32_t), h->stream));
            h->err = "recomputed transforms: a gradient block found no free scratch slot";
            return RDXG_ERR_CUDA;
        }
    }
    if (!h->dTcStatus) return RDXG_OK;
    int32_t st = 0;
    CK(h, cudaMemcpyAsync(&st, h->dTcStatus, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if (st == 0) return RDXG_OK;
    CK(h, cudaMemsetAsync(h->dTcStatus, 0, sizeof(int32_t), h->stream));
    h->err = std::string("tensor-core mode expansion: ") +
             (st == 1 ? "the mode tile copy" : "the products") + " did not complete within the wait limit";
    return RDXG_ERR_CUDA;
}

// finite-difference gradient of the patches in the FD list
void launch_fd(rdxg_solver* h, cudaStream_t st) {
    if (h->fusedFd) {
        with_eval(h->N, [&](auto E) {
            EvalParams<float> e = make_evalparams<float>(h);
            decltype(E)::fd_half(e, h->numSMs, st);
        });
        return;
    }
    with_size(h->N, h->fp64, [&](auto L, auto t) {
        using T = decltype(t);
        KParams<T> kp = make_kparams<T>(h);
        decltype(L)::fd(kp, h->fdGrid, h->M, st);
    });
}
void launch_fd(rdxg_solver* h) { launch_fd(h, h->stream); }

// FP32 map of metric requests (the point as float in dynamic shared memory, under 44 KB);
// RDXG_MAP64=1: the FP64 map for metric requests too (precision studies)
int cg_x1smem(const rdxg_solver* h) {
    const char* m64 = getenv("RDXG_MAP64");
    if (m64 && atoi(m64)) return 0;
    return (!h->fp64 && (size_t)h->nFree * sizeof(float) <= 44 * 1024) ? 1 : 0;
}

// The solver kernel's form: staged when the patch's data fit in kCgStageBytes (the null-space
// map too when it fits beside them), unless pinned to the global-memory form
// (rdxg_set_launch_shape, or RDXG_CG_STAGE=0 in the environment).
void cg_stage_choice(const rdxg_solver* h, int32_t* stage, int32_t* map, size_t* bytes) {
    const char* cs = getenv("RDXG_CG_STAGE");
    const bool allow = h->cgForm != 2 && !(cs && !atoi(cs));
    const int nT = h->fused ? h->nTilesH : h->nTiles;
    int m = cg_x1smem(h);
    size_t b = CgStageLayout(h->nFree, h->nObj, nT, m, h->nPar, h->I, h->mapMaxNnz).total;
    if (m && b > kCgStageBytes) {
        m = 0;
        b = CgStageLayout(h->nFree, h->nObj, nT, 0, h->nPar, h->I, h->mapMaxNnz).total;
    }
    *stage = (allow && b <= kCgStageBytes) ? 1 : 0;
    *map = *stage ? m : 0;
    *bytes = b;
}

template <typename T>
CgArgs<T> make_cgargs(rdxg_solver* h, const CgParams& prm) {
    CgArgs<T> a{};
    a.prm = prm;
    a.P = h->P; a.I = h->I; a.M = h->M; a.nObj = h->nObj; a.nPar = h->nPar; a.nTiles = h->nTiles; a.ps = h->ps;
    a.states = h->dStates; a.vec = h->dVec; a.metrics = h->dMetrics; a.alpha = h->dAlpha; a.alphaOff = h->dAlphaOff;
    a.alphaOffF = h->dAlphaOffF;
    a.galpha = h->dGalpha; a.partial = h->dPartial; a.objWeight = h->dObjW;
    a.pgeo = h->dPGeo;
    a.rowPtr = h->dRowPtr; a.rowCol = h->dRowCol; a.rowVal = h->dRowVal; a.rowVal32 = h->dRowVal32;
    a.colPtr = h->dColPtr; a.colRow = h->dColRow; a.colVal = h->dColVal;
    a.curTilt = h->dCurTilt; a.resAlpha = h->dResAlpha; a.tiltX = h->geo.tilt_x; a.tiltY = h->geo.tilt_y;
    a.alphaEff = (T*)h->dAlphaEff; a.req = h->dReq; a.gmethod = h->dGm; a.modeCount = h->dMc; a.active = h->dActive;
    a.fused = h->fused ? 1 : 0;
    a.x1Smem = cg_x1smem(h);
    a.stage = h->cgStage; a.stageMap = h->cgStageMap; a.maxNnz = h->mapMaxNnz;
    a.objMetric = h->dObjMetric; a.L = make_lists(h); a.nTilesH = h->nTilesH;
    a.chunkSize = h->chunk; a.chunksPerPatch = h->chunksPerPatch; a.objChunk0 = h->dPObjChunk0;
    a.objFirst = h->dPObjFirst; a.objCount = h->dPObjCount; a.aux = h->dAux;
    a.regW = h->hRegW.empty() ? nullptr : h->dRegW;
    a.phaseList = (!h->fused && h->tcPlan.valid) ? 1 : 0;
    return a;
}

template <typename T>
int create_static(rdxg_solver* h, const rdxg_static* s) {
    const int n = h->n, N = h->N, M = h->M, C = h->C;
    const size_t n2 = (size_t)n * n, N2 = (size_t)N * N;
    std::vector<T> Z(M * n2), A(n2, (T)0), phi(C * n2), cn(C);
    for (size_t i = 0; i < M * n2; ++i) Z[i] = (T)s->modes[i];
    double a2 = 0, area = 0;
    for (int k = 0; k < s->n_pupil_support; ++k) {
        const int q = s->pupil_support[k];
        if (q < 0 || (size_t)q >= n2) { h->err = "pupil_support index out of range"; return RDXG_ERR_ARG; }
        A[q] = (T)s->pupil[q];
        a2 += s->pupil[q] * s->pupil[q];
        area += s->pupil[q];
    }
    h->area = area;
    // Channel::initPatch: otfNormalization = 1/sqrt(max |OTF(phi = 0)|); the maximum is the
    // zero lag of the pupil autocorrelation, sum A^2 over the pupil support.
    for (int c = 0; c < C; ++c) cn[c] = (T)(1.0 / std::sqrt(a2));
    // the adjoint's factor per object and channel (project_modes): Vogel -2 area w^2 / N^6 / c
    // (X carries the factor c: the projection is c N^2 (G (*) PF)), exact gradient
    // -4 c^2 w / (ps^2 N^2) / c
    std::vector<double> gs(2 * (size_t)h->nObj * C);
    const double N2d = (double)N2;
    for (int o = 0; o < h->nObj; ++o)
        for (int c = 0; c < C; ++c) {
            const double cc = (double)cn[c], w = h->objWeight[o];
            gs[(size_t)o * C + c] = -2.0 * area * w * w / (N2d * N2d * N2d) / cc;
            gs[((size_t)h->nObj + o) * C + c] = -4.0 * cc * cc * w / ((double)h->ps * h->ps * N2d) / cc;
        }
    for (size_t i = 0; i < C * n2; ++i) phi[i] = (T)s->phi_fixed[i];
    std::vector<uint8_t> mask(N2, 0);
    for (int k = 0; k < s->n_otf_support; ++k) {
        const int u = s->otf_support[k];
        if (u < 0 || (size_t)u >= N2) { h->err = "otf_support index out of range"; return RDXG_ERR_ARG; }
        mask[u] = 1;
    }
    std::vector<cx<T>> tw(N);
    for (int k = 0; k < N; ++k) {
        const double ang = 2.0 * M_PI * (double)k / (double)N;
        tw[k].x = (T)std::cos(ang);
        tw[k].y = (T)(-std::sin(ang));
    }
    int r;
    if ((r = upload(h, &h->dZ, Z)) || (r = upload(h, &h->dA, A)) || (r = upload(h, &h->dPhi, phi)) ||
        (r = upload(h, &h->dOtfNorm, cn)) || (r = upload(h, &h->dTw, tw)))
        return r;
    void* v;
    if ((r = upload(h, &v, mask))) return r;
    h->dMask = (uint8_t*)v;
    if ((r = upload(h, &v, gs))) return r;
    h->dGradScale = (double*)v;
    return RDXG_OK;
}

template <typename T>
int alloc_patch_buffers(rdxg_solver* h) {
    const size_t P = h->Pmax, I = h->I, N2 = (size_t)h->N * h->N, n2 = (size_t)h->n * h->n;
    const size_t G = P * I, PO = P * h->nObj;
    int r;
    if ((r = dalloc_t(h, &h->dCut, G * h->cs * h->cs)) || (r = dalloc_t(h, &h->dShift, G * 2)) ||
        (r = dalloc_t(h, &h->dMean, G)) || (r = dalloc_t(h, &h->dStd, G)) || (r = dalloc_t(h, &h->dNoise, G)) ||
        (r = dalloc_t(h, &h->dRg, G)) || (r = dalloc(h, &h->dAlphaEff, G * h->M * sizeof(T))) ||
        (r = dalloc(h, &h->dD, G * N2 * sizeof(cx<T>))) ||
        (r = dalloc(h, &h->dO, PO * N2 * sizeof(cx<T>))) || (r = dalloc(h, &h->dQt, PO * N2 * sizeof(T))) ||
        (r = dalloc_t(h, &h->dGamma, PO)) || (r = dalloc_t(h, &h->dPartial, PO * h->nTiles)) ||
        (r = dalloc_t(h, &h->dGalpha, G * h->M)) || (r = dalloc_t(h, &h->dReq, P)) ||
        (r = dalloc_t(h, &h->dGm, P)) || (r = dalloc_t(h, &h->dMc, P)) || (r = dalloc_t(h, &h->dReinit, G)) ||
        (r = dalloc_t(h, &h->dCurTilt, G * 2)) || (r = dalloc_t(h, &h->dResAlpha, G * 2)) ||
        (r = dalloc_t(h, &h->dStates, P)) || (r = dalloc_t(h, &h->dVec, P * 5 * h->nFree)) ||
        (r = dalloc_t(h, &h->dAlpha, P * h->nPar)) || (r = dalloc_t(h, &h->dAlphaOff, P * h->nPar)) ||
        (r = dalloc_t(h, &h->dAlphaOffF, P * h->nPar)) ||
        (r = dalloc_t(h, &h->dActive, 1)) || (r = dalloc_t(h, &h->dGradP, P)) || (r = dalloc_t(h, &h->dFdP, P)) ||
        (r = dalloc_t(h, &h->dEvalP, P)) || (r = dalloc_t(h, &h->dCounters, kNumCounters)))
        return r;
    CK(h, cudaMemset(h->dCounters, 0, kNumCounters * sizeof(int32_t)));
    CK(h, cudaMallocHost((void**)&h->hActive, sizeof(int32_t)));
    CK(h, cudaMemset(h->dReinit, 0, G));
    return RDXG_OK;
}

// Bytes of the per-image transforms kept from an evaluation for the gradient kernels: X and PF
// of every image, and S where it is needed only by them (the fused path, whose evaluation
// keeps no full OTF otherwise); and of the scratch that replaces them when recomputed.
size_t kept_transform_bytes(const rdxg_solver* h) {
    const size_t G = (size_t)h->Pmax * h->I, cxs = h->fp64 ? 16 : 8;
    const size_t N2 = (size_t)h->N * h->N, n2 = (size_t)h->n * h->n;
    return G * cxs * (N2 + n2 + (h->fused ? N2 : 0));
}
size_t recompute_scratch_bytes(const rdxg_solver* h) {
    return (size_t)h->nsmid * h->slotsPerSM * h->N * h->N * (h->fp64 ? 16 : 8) + (size_t)h->nsmid * sizeof(unsigned);
}

// Allocates (or frees) the kept transforms and the recomputation scratch for the mode chosen.
int setup_transforms(rdxg_solver* h, bool recompute) {
    const size_t G = (size_t)h->Pmax * h->I, cxs = h->fp64 ? 16 : 8;
    const size_t N2 = (size_t)h->N * h->N, n2 = (size_t)h->n * h->n;
    int r;
    if (recompute) {
        if (h->scrBlocks < 1) {
            h->err = "recomputed transforms: the recomputing kernels do not fit this size's shared memory";
            return RDXG_ERR_UNSUPPORTED;
        }
        dfree(h, &h->dX, G * N2 * cxs);
        dfree(h, &h->dPF, G * n2 * cxs);
        if (h->fused) dfree(h, &h->dS, G * N2 * cxs);
        const size_t tiles = (size_t)h->nsmid * h->slotsPerSM * N2 * cxs;
        if (!h->dXscr && (r = dalloc(h, &h->dXscr, tiles))) return r;
        if (!h->dSlotMask) {
            if ((r = dalloc_t(h, &h->dSlotMask, (size_t)h->nsmid))) return r;
            CK(h, cudaMemsetAsync(h->dSlotMask, 0, (size_t)h->nsmid * sizeof(unsigned), h->stream));
        }
        if (!h->dRcStatus) {
            if ((r = dalloc_t(h, &h->dRcStatus, 1))) return r;
            CK(h, cudaMemsetAsync(h->dRcStatus, 0, sizeof(int32_t), h->stream));
        }
        CK(h, cudaStreamSynchronize(h->stream));
    } else {
        dfree(h, &h->dXscr, (size_t)h->nsmid * h->slotsPerSM * N2 * cxs);
        dfree(h, &h->dSlotMask, (size_t)h->nsmid * sizeof(unsigned));
        if (!h->dX && (r = dalloc(h, &h->dX, G * N2 * cxs))) return r;
        if (!h->dPF && (r = dalloc(h, &h->dPF, G * n2 * cxs))) return r;
    }
    // the general path's per-object accumulation reads S in every round
    if ((!recompute || !h->fused) && !h->dS && (r = dalloc(h, &h->dS, G * N2 * cxs))) return r;
    h->recompute = recompute;
    return RDXG_OK;
}

// The maps of a shape in the handle's layout (row = image slot * M + mode), both ways, from
// entries whose rows are in the shape's own layout (packed image k * nMode + mode).
int shape_maps(rdxg_solver* h, rdxg_solver::Shape& sh, int64_t nnz, const int32_t* rows, const int32_t* cols,
               const double* vals) {
    const int nPar = h->nPar, nF = sh.nFree, Ms = sh.M;
    std::vector<int32_t> hr(nnz);
    for (int64_t e = 0; e < nnz; ++e) {
        const int r = rows[e], c = cols[e];
        if (r < 0 || r >= sh.nImg * Ms || c < 0 || c >= nF) { h->err = "null-space entry out of range"; return RDXG_ERR_ARG; }
        hr[e] = (r / Ms) * h->M + r % Ms;
    }
    std::vector<int32_t>& rc = sh.rowPtr;
    std::vector<int32_t>& cc = sh.colPtr;
    rc.assign(nPar + 1, 0);
    cc.assign(nF + 1, 0);
    for (int64_t e = 0; e < nnz; ++e) {
        rc[hr[e] + 1]++;
        cc[cols[e] + 1]++;
    }
    for (int i = 0; i < nPar; ++i) rc[i + 1] += rc[i];
    for (int i = 0; i < nF; ++i) cc[i + 1] += cc[i];
    sh.rowCol.assign(nnz, 0); sh.colRow.assign(nnz, 0);
    sh.rowVal.assign(nnz, 0.0); sh.colVal.assign(nnz, 0.0);
    std::vector<int32_t> rfill(rc.begin(), rc.end() - 1), cfill(cc.begin(), cc.end() - 1);
    for (int64_t e = 0; e < nnz; ++e) {
        const int r = hr[e], c = cols[e];
        sh.rowCol[rfill[r]] = c; sh.rowVal[rfill[r]++] = vals[e];
        sh.colRow[cfill[c]] = r; sh.colVal[cfill[c]++] = vals[e];
    }
    return RDXG_OK;
}

// The image and object tables of a shape: each channel's first `frames` images (all when
// frames < 0), in the handle's image order, packed into the first slots.
int shape_tables(rdxg_solver* h, rdxg_solver::Shape& sh) {
    std::vector<int> rank(h->C, 0);
    sh.imgObj.assign(h->I, 0);
    sh.imgCh.assign(h->I, 0);
    int k = 0;
    for (int j = 0; j < h->I; ++j) {
        const int c = h->imgCh[j];
        if (sh.frames < 0 || rank[c] < sh.frames) {
            sh.imgObj[k] = h->imgObj[j];
            sh.imgCh[k] = c;
            ++k;
        }
        rank[c]++;
    }
    sh.nImg = k;
    sh.objFirst.assign(h->nObj, -1);
    sh.objCount.assign(h->nObj, 0);
    for (int j = 0; j < sh.nImg; ++j) {
        const int o = sh.imgObj[j];
        if (sh.objFirst[o] < 0) sh.objFirst[o] = j;
        sh.objCount[o]++;
    }
    for (int o = 0; o < h->nObj; ++o)
        if (sh.objCount[o] == 0) { h->err = "patch shape: an object without images"; return RDXG_ERR_ARG; }
    sh.objChunk0.assign(h->nObj, 0);
    int c0 = 0;
    for (int o = 0; o < h->nObj; ++o) {
        sh.objChunk0[o] = c0;
        c0 += (sh.objCount[o] + h->chunk - 1) / h->chunk;
    }
    sh.chunks = c0;
    return RDXG_OK;
}

int build_nullspace(rdxg_solver* h, const rdxg_static* s) {
    h->shapes.assign(1, rdxg_solver::Shape{});
    rdxg_solver::Shape& sh = h->shapes[0];
    sh.frames = -1; sh.M = h->M; sh.nFree = h->nFree; sh.nImg = h->I;
    return shape_maps(h, sh, s->ns_nnz, s->ns_rows, s->ns_cols, s->ns_vals);
}

// Uploads every patch's geometry and tables (patches without a shape take shape 0) and the
// maps of every shape, one after the other.
int upload_geometry(rdxg_solver* h) {
    for (rdxg_solver::Shape& sh : h->shapes) {
        int r = shape_tables(h, sh);
        if (r) return r;
    }
    const size_t P = h->Pmax;
    h->patchShape.resize(P, 0);
    std::vector<int32_t> rowPtr, rowCol, colPtr, colRow;
    std::vector<double> rowVal, colVal;
    std::vector<int> rowBase(h->shapes.size()), colBase(h->shapes.size());
    for (size_t k = 0; k < h->shapes.size(); ++k) {
        const rdxg_solver::Shape& sh = h->shapes[k];
        const int32_t off = (int32_t)rowCol.size();
        rowBase[k] = (int)rowPtr.size();
        colBase[k] = (int)colPtr.size();
        for (int32_t v : sh.rowPtr) rowPtr.push_back(v + off);
        for (int32_t v : sh.colPtr) colPtr.push_back(v + off);
        rowCol.insert(rowCol.end(), sh.rowCol.begin(), sh.rowCol.end());
        colRow.insert(colRow.end(), sh.colRow.begin(), sh.colRow.end());
        rowVal.insert(rowVal.end(), sh.rowVal.begin(), sh.rowVal.end());
        colVal.insert(colVal.end(), sh.colVal.begin(), sh.colVal.end());
    }
    std::vector<PatchGeo> geo(P);
    std::vector<int32_t> io(P * h->I), ic(P * h->I), of(P * h->nObj), oc(P * h->nObj), ch0(P * h->nObj);
    for (size_t p = 0; p < P; ++p) {
        const int k = h->patchShape[p];
        const rdxg_solver::Shape& sh = h->shapes[k];
        geo[p] = PatchGeo{sh.nImg, sh.M, sh.nFree, sh.chunks, rowBase[k], colBase[k]};
        std::copy(sh.imgObj.begin(), sh.imgObj.end(), io.begin() + p * h->I);
        std::copy(sh.imgCh.begin(), sh.imgCh.end(), ic.begin() + p * h->I);
        std::copy(sh.objFirst.begin(), sh.objFirst.end(), of.begin() + p * h->nObj);
        std::copy(sh.objCount.begin(), sh.objCount.end(), oc.begin() + p * h->nObj);
        std::copy(sh.objChunk0.begin(), sh.objChunk0.end(), ch0.begin() + p * h->nObj);
    }
    int r;
    if (!h->dPGeo) {
        if ((r = dalloc_t(h, &h->dPGeo, P)) || (r = dalloc_t(h, &h->dPImgObj, P * h->I)) ||
            (r = dalloc_t(h, &h->dPImgCh, P * h->I)) || (r = dalloc_t(h, &h->dPObjFirst, P * h->nObj)) ||
            (r = dalloc_t(h, &h->dPObjCount, P * h->nObj)) || (r = dalloc_t(h, &h->dPObjChunk0, P * h->nObj)))
            return r;
    }
    CK(h, cudaMemcpy(h->dPGeo, geo.data(), P * sizeof(PatchGeo), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dPImgObj, io.data(), io.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dPImgCh, ic.data(), ic.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dPObjFirst, of.data(), of.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dPObjCount, oc.data(), oc.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dPObjChunk0, ch0.data(), ch0.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    h->mapMaxNnz = 0;
    for (const rdxg_solver::Shape& sh : h->shapes) h->mapMaxNnz = std::max(h->mapMaxNnz, (int32_t)sh.rowCol.size());
    // the maps (reallocated when their sizes change)
    const size_t nnz = rowCol.size();
    if (rowPtr.size() != h->mapRowEntries || colPtr.size() != h->mapColEntries || nnz != h->mapNnz) {
        dfree(h, &h->dRowPtr, h->mapRowEntries * sizeof(int32_t));
        dfree(h, &h->dColPtr, h->mapColEntries * sizeof(int32_t));
        dfree(h, &h->dRowCol, h->mapNnz * sizeof(int32_t));
        dfree(h, &h->dColRow, h->mapNnz * sizeof(int32_t));
        dfree(h, &h->dRowVal, h->mapNnz * sizeof(double));
        dfree(h, &h->dColVal, h->mapNnz * sizeof(double));
        dfree(h, &h->dRowVal32, h->mapNnz * sizeof(float));
        if ((r = dalloc_t(h, &h->dRowPtr, rowPtr.size())) || (r = dalloc_t(h, &h->dColPtr, colPtr.size())) ||
            (r = dalloc_t(h, &h->dRowCol, nnz)) || (r = dalloc_t(h, &h->dColRow, nnz)) ||
            (r = dalloc_t(h, &h->dRowVal, nnz)) || (r = dalloc_t(h, &h->dColVal, nnz)) ||
            (r = dalloc_t(h, &h->dRowVal32, nnz)))
            return r;
        h->mapRowEntries = rowPtr.size();
        h->mapColEntries = colPtr.size();
        h->mapNnz = nnz;
    }
    std::vector<float> rowVal32(rowVal.begin(), rowVal.end());
    CK(h, cudaMemcpy(h->dRowPtr, rowPtr.data(), rowPtr.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dColPtr, colPtr.data(), colPtr.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dRowCol, rowCol.data(), nnz * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dColRow, colRow.data(), nnz * sizeof(int32_t), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dRowVal, rowVal.data(), nnz * sizeof(double), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dColVal, colVal.data(), nnz * sizeof(double), cudaMemcpyHostToDevice));
    CK(h, cudaMemcpy(h->dRowVal32, rowVal32.data(), nnz * sizeof(float), cudaMemcpyHostToDevice));
    return RDXG_OK;
}

// Arguments of the re-shifts (SubImage::adjustShifts of patches that request one), done by the
// solver kernel in the rounds and by k_shift for the initial re-cut of a warm start.
ShiftArgs make_shift_args(rdxg_solver* h) {
    ShiftArgs sa{};
    sa.P = h->P; sa.I = h->I; sa.M = h->M; sa.nObj = h->nObj; sa.ps = h->ps; sa.cs = h->cs; sa.margin = h->margin;
    sa.tiltX = h->haveJ ? h->geo.tilt_x : -1; sa.tiltY = h->haveJ ? h->geo.tilt_y : -1;
    sa.req = h->dReq; sa.alpha = h->dAlpha; sa.tiltOff = h->dCurTilt; sa.shift = h->dShift;
    sa.reinit = h->dReinit; sa.imgObj = h->dPImgObj; sa.pgeo = h->dPGeo; sa.aux = h->fused ? h->dAux : nullptr;
    std::memcpy(sa.J, h->J, sizeof(sa.J));
    std::memcpy(sa.Jinv, h->Jinv, sizeof(sa.Jinv));
    return sa;
}

// (re)initialise the loaded patches: shifts 0 (or those of the initial coefficients), full
// image preparation, gamma
int prepare_patches(rdxg_solver* h) {
    const size_t G = (size_t)h->P * h->I;
    CK(h, cudaMemsetAsync(h->dShift, 0, G * 2 * sizeof(int32_t), h->stream));
    CK(h, cudaMemsetAsync(h->dCurTilt, 0, G * 2 * sizeof(double), h->stream));
    CK(h, cudaMemcpyAsync(h->dResAlpha, h->hResAlpha.data(), G * 2 * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (h->haveInit && h->initRecut) {
        // Solver::shiftAndInit(alpha_offset, true) after loadInit (solver.cpp:412-413): every
        // image's window follows the tilts of the initial coefficients (SubImage::adjustShifts)
        CK(h, cudaMemcpyAsync(h->dAlpha, h->dInitAlpha, G * h->M * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
        const std::vector<int32_t> shiftReq(h->P, REQ_SHIFT);
        CK(h, cudaMemcpyAsync(h->dReq, shiftReq.data(), h->P * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        launch_shift(make_shift_args(h), h->P, h->stream);
        h->launches++;
        CKL(h);
    }
    int rc = RDXG_OK;
    with_size(h->N, h->fp64, [&](auto L, auto t) {
        using T = decltype(t);
        KParams<T> kp = make_kparams<T>(h);
        if (h->fitPlane) launch_fit_plane<T>(kp, 1, h->P * h->nObj, h->stream);   // ObjectData::initPatch
        decltype(L)::prep(kp, 1, (int)G, h->stream);
    });
    h->launches += h->fitPlane ? 2 : 1;
    CKL(h);
    std::vector<double> rg(G);
    CK(h, cudaMemcpyAsync(rg.data(), h->dRg, G * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    // Object::addRegGamma (object.cpp:465-468): reg_gamma = sum_j 0.1 rg_j / nObjectImages
    std::vector<double> gam((size_t)h->P * h->nObj, 0.0);
    for (int p = 0; p < h->P; ++p) {
        const rdxg_solver::Shape& sh = h->shapes[h->patchShape[p]];
        for (int j = 0; j < sh.nImg; ++j) {
            const int o = sh.imgObj[j];
            gam[(size_t)p * h->nObj + o] += 0.10 * rg[(size_t)p * h->I + j] / sh.objCount[o];
        }
    }
    if (h->haveFixedGamma) gam = h->hFixedGamma;
    for (double g : gam) {
        if (!std::isfinite(g)) { h->err = "non-finite regularisation (image with zero variance?)"; rc = RDXG_ERR_NONFINITE; }
    }
    CK(h, cudaMemcpyAsync(h->dGamma, gam.data(), gam.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    h->dirty = false;
    return rc;
}

int set_patches_common(rdxg_solver* h, int32_t P, const double* residual_alpha, const double* fixed_gamma) {
    if (P < 1 || P > h->Pmax) { h->err = "n_patches out of range"; return RDXG_ERR_ARG; }
    if (h->ragged && P != h->raggedPatches) {
        h->err = "the patch shapes were given for " + std::to_string(h->raggedPatches) + " patches, not " +
                 std::to_string(P);
        return RDXG_ERR_ARG;
    }
    h->P = P;
    h->haveInit = false;     // a new batch starts at zero unless rdxg_set_initial_alpha follows
    const size_t G = (size_t)P * h->I;
    h->hResAlpha.assign(G * 2, 0.0);
    if (residual_alpha) std::memcpy(h->hResAlpha.data(), residual_alpha, G * 2 * sizeof(double));
    h->haveFixedGamma = fixed_gamma != nullptr;
    if (fixed_gamma) h->hFixedGamma.assign(fixed_gamma, fixed_gamma + (size_t)P * h->nObj);
    int r = prepare_patches(h);
    h->loaded = (r == RDXG_OK);
    return r;
}

// alpha_eff on the host for single evaluations
template <typename T>
int upload_alpha(rdxg_solver* h, const double* alpha) {
    const size_t G = (size_t)h->P * h->I;
    std::vector<double> curTilt(G * 2);
    CK(h, cudaMemcpyAsync(curTilt.data(), h->dCurTilt, G * 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    std::vector<T> ae(G * h->M);
    for (size_t g = 0; g < G; ++g) {
        // a ragged batch: the image slots and modes a patch does not use stay at zero
        const rdxg_solver::Shape& sh = h->shapes[h->patchShape[g / h->I]];
        const bool slotUsed = (int)(g % h->I) < sh.nImg;
        for (int m = 0; m < h->M; ++m) {
            if (!slotUsed || m >= sh.M) { ae[g * h->M + m] = (T)0; continue; }
            double v = alpha[g * h->M + m];
            if (m == h->geo.tilt_x) v += curTilt[g * 2 + 1] - h->hResAlpha[g * 2 + 1];
            else if (m == h->geo.tilt_y) v += curTilt[g * 2 + 0] - h->hResAlpha[g * 2 + 0];
            ae[g * h->M + m] = (T)v;
        }
    }
    CK(h, cudaMemcpyAsync(h->dAlphaEff, ae.data(), ae.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return RDXG_OK;
}

int metric_from_partials(rdxg_solver* h, double* metric) {
    const size_t PO = (size_t)h->P * h->nObj;
    std::vector<double> part(PO * h->nTiles);
    CK(h, cudaMemcpyAsync(part.data(), h->dPartial, part.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int p = 0; p < h->P; ++p) {
        double sum = 0;
        for (int o = 0; o < h->nObj; ++o) {
            if (h->objWeight[o] == 0.0) continue;
            double m = 0;
            for (int t = 0; t < h->nTiles; ++t) m += part[((size_t)p * h->nObj + o) * h->nTiles + t];
            sum += h->objWeight[o] * (m / ((double)h->ps * h->ps));
        }
        metric[p] = sum;
    }
    return RDXG_OK;
}

int set_requests(rdxg_solver* h, int req, int gm, int mc) {
    std::vector<int32_t> a(h->P, req), b(h->P, gm), c(h->P, mc), all(h->P);
    for (int p = 0; p < h->P; ++p) {
        all[p] = p;
        c[p] = std::min(mc, h->shapes[h->patchShape[p]].M);   // a ragged batch: the patch's own modes
    }
    int32_t cnt[2] = {0, 0};
    if (req == REQ_DF) { if (gm == GM_FD) cnt[1] = h->P; else cnt[0] = h->P; }
    CK(h, cudaMemcpyAsync(h->dGradP, all.data(), h->P * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dFdP, all.data(), h->P * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dCounters + 2, cnt, 2 * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dReq, a.data(), h->P * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dGm, b.data(), h->P * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dMc, c.data(), h->P * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    if (!h->fused) {
        // the general path's tensor-core expansion takes the patches of this evaluation: all
        const int32_t nP = h->P;
        CK(h, cudaMemcpyAsync(h->dEvalP, all.data(), h->P * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaMemcpyAsync(h->dCounters + 4, &nP, sizeof(nP), cudaMemcpyHostToDevice, h->stream));
    }
    CK(h, cudaStreamSynchronize(h->stream));
    return RDXG_OK;
}

// The mode expansion of the general path on the tensor cores (FP32 handles whose shape the
// tensor-core kernel takes): the phases of the listed patches' images, which k_forward and
// the recomputing gradient kernels then read instead of expanding the modes themselves.
void phase_general(rdxg_solver* h, cudaStream_t st) {
    if (h->fused || !h->tcPlan.valid) return;
    PhaseTcArgs a;
    a.Zt = h->dZt; a.alphaEff = (const float*)h->dAlphaEff; a.phiFixed = (const float*)h->dPhi;
    a.imgCh = h->dPImgCh; a.evalP = h->dEvalP; a.nEvalP = h->dCounters + kCounterEvalP;
    a.phi = (float*)h->dPhiImg; a.status = h->dTcStatus;
    a.I = h->I; a.M = h->M; a.n2 = h->n * h->n; a.nCh = h->C;
    a.G = h->tcPlan.G; a.NT = h->tcPlan.NT; a.KP = h->tcPlan.KP; a.parts = h->tcPlan.parts;
    launch_phase_tc(a, h->tcPlan, st);
}

CgParams make_cg_params(rdxg_solver* h, const rdxg_solve_params* s) {
    CgParams prm{};
    prm.n_free = h->nFree;
    prm.n_modes = h->M;
    prm.mode_start = s->mode_start > 0 ? s->mode_start : 1;
    prm.mode_step = s->mode_step > 0 ? s->mode_step : 1;
    prm.max_iterations = s->max_iterations;
    prm.min_iterations = s->min_iterations;
    prm.target_iterations = s->target_iterations;
    prm.fd_first = s->fd_first;
    prm.max_fails = 3;
    prm.max_metrics = s->max_metrics > 0 ? s->max_metrics : 1;
    prm.ftol = s->ftol;
    prm.eps = s->eps;
    const double nTotalPixels = (double)h->I * h->ps * h->ps;
    prm.grad_scale = 1.0 / (nTotalPixels * nTotalPixels);
    prm.brent_tol = 0.1;
    prm.init_step = 1E-21;
    return prm;
}

// Half-plane of the OTF support and buffers of the fused evaluation path.
int setup_fused(rdxg_solver* h, const rdxg_static* s) {
    const int N = h->N;
    h->fused = false;
    h->fusedFd = false;
    if (h->fp64 || !(N == 32 || N == 64 || N == 88)) return RDXG_OK;
    std::vector<uint8_t> mask((size_t)N * N, 0);
    for (int k = 0; k < s->n_otf_support; ++k) mask[s->otf_support[k]] = 1;
    h->hIdx.clear();
    for (int c = 0; c < N * N; ++c) {
        if (!mask[c]) continue;
        const int cy = c / N, cx = c % N;
        if (cy == 0 || cx == 0) return RDXG_OK;                  // Nyquist terms: use the general path
        if (!mask[(N - cy) * N + (N - cx)]) return RDXG_OK;      // not symmetric: general path
        // half plane along x: its points sit in the un-centred columns [0, N/2)
        if (cx > N / 2 || (cx == N / 2 && cy >= N / 2)) h->hIdx.push_back(c);
    }
    h->nH = (int)h->hIdx.size();
    h->hPos.resize(h->nH);
    for (int k = 0; k < h->nH; ++k) {
        const int c = h->hIdx[k];
        h->hPos[k] = (((c / N) + N / 2) % N) * (N + 1) + ((c % N) + N / 2) % N;
    }
    h->nTilesH = (h->nH + kReduceTile - 1) / kReduceTile;
    h->npt = 1;
    if (h->nH > N * (N / 2 + 1)) return RDXG_OK;   // more points than the staging area holds
    // more points than the evaluation's register accumulators hold
    if (h->nH > (N == 32 ? kFusedMaxPoints<32>::value : N == 64 ? kFusedMaxPoints<64>::value
                                                                 : kFusedMaxPoints<88>::value))
        return RDXG_OK;
    const size_t smem = N == 32 ? EvalLauncher<float, 32>::smem(h->M, h->nH)
                      : N == 64 ? EvalLauncher<float, 64>::smem(h->M, h->nH)
                                : EvalLauncher<float, 88>::smem(h->M, h->nH);
    if (smem > 227 * 1024) return RDXG_OK;   // does not fit
    h->chunk = h->geo.eval_chunk > 0 ? h->geo.eval_chunk : 6;
    h->objChunk0.assign(h->nObj, 0);
    int c0 = 0;
    for (int o = 0; o < h->nObj; ++o) {
        h->objChunk0[o] = c0;
        c0 += (h->objCount[o] + h->chunk - 1) / h->chunk;
    }
    h->chunksPerPatch = c0;
    const size_t P = h->Pmax, G = P * h->I, PO = P * h->nObj;
    int r;
    void* v;
    if ((r = upload(h, &v, h->hIdx))) return r;
    h->dHIdx = (int32_t*)v;
    if ((r = upload(h, &v, h->objChunk0))) return r;
    h->dObjChunk0 = (int32_t*)v;
    if ((r = upload(h, &v, h->hPos))) return r;
    h->dHPos = (int32_t*)v;
    if ((r = dalloc(h, &h->dDh, G * h->nH * sizeof(float2))) || (r = dalloc(h, &h->dOh, PO * h->nH * sizeof(float2))) ||
        (r = dalloc(h, &h->dPart, P * h->chunksPerPatch * 4 * (size_t)h->nH * sizeof(float))) ||
        (r = dalloc_t(h, &h->dObjMetric, PO * h->nTilesH)) || (r = dalloc_t(h, &h->dEval, P * h->chunksPerPatch)) ||
        (r = dalloc_t(h, &h->dPoList, PO)) || (r = dalloc_t(h, &h->dAux, P * 2)) ||
        (r = dalloc(h, &h->dPhiImg, G * (size_t)h->n * h->n * sizeof(float))))
        return r;
    cudaError_t e = cudaSuccess;
    int occ = 0;
    with_eval(N, [&](auto L) {
        e = decltype(L)::setup(h->M, h->npt, h->nH);
        occ = decltype(L)::occupancy(h->M, h->npt, h->nH);
    });
    if (e != cudaSuccess) { h->err = std::string("fused setup: ") + cudaGetErrorString(e); return RDXG_ERR_CUDA; }
    if (occ < 1) occ = 1;
    size_t fdSmem = 0;
    with_eval(N, [&](auto L) { fdSmem = decltype(L)::fd_smem(h->nH); });
    h->fusedFd = fdSmem + 1024 <= kMaxSmem;   // 1 KB left for static shared memory
    h->evalGrid = h->numSMs * occ;
    h->reduceGrid = h->numSMs * 8;
    h->phaseGrid = h->numSMs * 4;
    h->fused = true;
    const char* pm = getenv("RDXG_PHASE_PARTS");
    const int parts = pm ? atoi(pm) : 3;
    return setup_phase_tc(h, parts == 0 || parts == 2 ? parts : 3);
}

// evaluation work lists built on the host for single evaluations of every patch
int host_lists(rdxg_solver* h, int req, int mode) {
    std::vector<EvalItem> ev;
    std::vector<PoItem> po;
    for (int p = 0; p < h->P; ++p) {
        const rdxg_solver::Shape& sh = h->shapes[h->patchShape[p]];
        for (int o = 0; o < h->nObj; ++o) {
            const int cnt = sh.objCount[o];
            const int nc = (cnt + h->chunk - 1) / h->chunk;
            for (int c = 0; c < nc; ++c) {
                EvalItem it;
                it.p = p; it.o = o; it.first = sh.objFirst[o] + c * h->chunk;
                it.count = std::min(h->chunk, cnt - c * h->chunk);
                it.chunk = sh.objChunk0[o] + c; it.df = req == REQ_DF ? 1 : 0;
                ev.push_back(it);
            }
            PoItem pi;
            pi.p = p; pi.o = o; pi.mode = mode;
            po.push_back(pi);
        }
    }
    std::vector<int32_t> pl(h->P);
    for (int p = 0; p < h->P; ++p) pl[p] = p;
    int32_t cnt[2] = {(int32_t)ev.size(), (int32_t)po.size()};
    const int32_t nP = h->P;
    CK(h, cudaMemcpyAsync(h->dEval, ev.data(), ev.size() * sizeof(EvalItem), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dPoList, po.data(), po.size() * sizeof(PoItem), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dEvalP, pl.data(), pl.size() * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dCounters, cnt, sizeof(cnt), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaMemcpyAsync(h->dCounters + 4, &nP, sizeof(nP), cudaMemcpyHostToDevice, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return RDXG_OK;
}

// Single evaluations (metric, gradient, restoration) on the fused path start from a zero
// reference object, so that their result depends on the point and the loaded patches only,
// not on what an earlier call left behind (the evaluation is exact for any reference object,
// but its rounding is not).
int reset_reference(rdxg_solver* h) {
    if (h->fused)
        CK(h, cudaMemsetAsync(h->dOh, 0, (size_t)h->P * h->nObj * h->nH * sizeof(float2), h->stream));
    return RDXG_OK;
}

int fused_pass(rdxg_solver* h, int req, int mode) {
    int r;
    if ((r = host_lists(h, req, mode))) return r;
    with_eval(h->N, [&](auto L) {
        EvalParams<float> e = make_evalparams<float>(h);
        decltype(L)::phase(e, h->phaseGrid, h->stream);
        decltype(L)::eval(e, h->npt, h->evalGrid, h->stream);
        decltype(L)::reduce(e, h->reduceGrid, h->stream);
    });
    CKL(h);
    return RDXG_OK;
}

int metric_from_objects(rdxg_solver* h, double* metric) {
    const size_t PO = (size_t)h->P * h->nObj;
    std::vector<double> om(PO * h->nTilesH);
    CK(h, cudaMemcpyAsync(om.data(), h->dObjMetric, om.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    for (int p = 0; p < h->P; ++p) {
        double sum = 0;
        for (int o = 0; o < h->nObj; ++o) {
            if (h->objWeight[o] == 0.0) continue;
            double m = 0;
            for (int t = 0; t < h->nTilesH; ++t) m += om[((size_t)p * h->nObj + o) * h->nTilesH + t];
            sum += h->objWeight[o] * (m / ((double)h->ps * h->ps));
        }
        metric[p] = sum;
    }
    return RDXG_OK;
}

}  // namespace

extern "C" {

int rdxg_version(void) { return 100; }

const char* rdxg_last_error(const rdxg_solver* h) { return h ? h->err.c_str() : "null handle"; }

int rdxg_create(const rdxg_geometry* g, const rdxg_static* s, rdxg_solver** out) {
    if (!g || !s || !out) return RDXG_ERR_ARG;
    *out = nullptr;
    rdxg_solver* h = new rdxg_solver();
    h->geo = *g;
    h->N = g->otf_size; h->n = g->pupil_pixels; h->ps = g->patch_size; h->M = g->n_modes;
    h->I = g->n_images; h->nObj = g->n_objects; h->C = g->n_channels; h->nFree = g->n_free;
    h->cs = g->cutout_size > 0 ? g->cutout_size : g->patch_size;
    h->margin = (h->cs - h->ps) / 2;
    h->nPar = h->I * h->M;
    h->Pmax = g->max_patches;
    h->fp64 = g->precision == RDXG_FP64;
    auto fail = [&](int code, const char* msg) {
        if (msg) h->err = msg;
        *out = h;          // hand the handle back so the caller can read the message
        return code;
    };
    if (h->N != 2 * h->n) return fail(RDXG_ERR_ARG, "otf_size must be 2 * pupil_pixels");
    if (g->eval_chunk < 0 || g->eval_chunk > kMaxChunk)
        return fail(RDXG_ERR_ARG, ("eval_chunk must be 0.." + std::to_string(kMaxChunk)).c_str());
    if (!supported_N(h->N)) return fail(RDXG_ERR_UNSUPPORTED, "otf_size not compiled (supported: 32, 64, 88, 128)");
    if (h->ps != h->N) return fail(RDXG_ERR_UNSUPPORTED, "patch_size must equal otf_size");
    if (h->cs < h->ps || ((h->cs - h->ps) & 1)) return fail(RDXG_ERR_ARG, "bad cutout_size");
    if (h->M < 1 || h->I < 1 || h->nObj < 1 || h->nObj > 64 || h->C < 1 || h->Pmax < 1 || h->nFree < 1)
        return fail(RDXG_ERR_ARG, "bad geometry");
    h->imgObj.assign(s->image_object, s->image_object + h->I);
    h->imgCh.assign(s->image_channel, s->image_channel + h->I);
    h->objFirst.assign(h->nObj, -1);
    h->objCount.assign(h->nObj, 0);
    for (int j = 0; j < h->I; ++j) {
        const int o = h->imgObj[j];
        if (o < 0 || o >= h->nObj || h->imgCh[j] < 0 || h->imgCh[j] >= h->C) return fail(RDXG_ERR_ARG, "bad image map");
        if (h->objFirst[o] < 0) h->objFirst[o] = j;
        if (h->objFirst[o] + h->objCount[o] != j) return fail(RDXG_ERR_ARG, "images of an object must be contiguous");
        h->objCount[o]++;
    }
    for (int o = 0; o < h->nObj; ++o)
        if (h->objCount[o] == 0) return fail(RDXG_ERR_ARG, "object without images");
    h->objWeight.assign(s->object_weight, s->object_weight + h->nObj);
    h->gradStep.assign(s->object_grad_step, s->object_grad_step + h->nObj);
    if (s->tilt_jacobian) {
        h->haveJ = true;
        h->J[0][0] = s->tilt_jacobian[0]; h->J[0][1] = s->tilt_jacobian[1];
        h->J[1][0] = s->tilt_jacobian[2]; h->J[1][1] = s->tilt_jacobian[3];
        const double det = h->J[0][0] * h->J[1][1] - h->J[0][1] * h->J[1][0];
        h->Jinv[0][0] = h->J[1][1] / det; h->Jinv[0][1] = -h->J[0][1] / det;
        h->Jinv[1][0] = -h->J[1][0] / det; h->Jinv[1][1] = h->J[0][0] / det;
    }
    h->nTiles = (h->N * h->N + kAccumThreads - 1) / kAccumThreads;
    cudaError_t e = cudaSetDevice(g->device);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); *out = h; return RDXG_ERR_CUDA; }
    e = cudaStreamCreateWithFlags(&h->own, cudaStreamNonBlocking);
    if (e != cudaSuccess) { h->err = cudaGetErrorString(e); *out = h; return RDXG_ERR_CUDA; }
    h->stream = h->own;
    int r = h->fp64 ? create_static<double>(h, s) : create_static<float>(h, s);
    if (!r) r = build_nullspace(h, s);
    if (!r) r = h->fp64 ? alloc_patch_buffers<double>(h) : alloc_patch_buffers<float>(h);
    std::vector<double> win(s->window, s->window + (size_t)h->ps * h->ps), nwin(s->noise_window, s->noise_window + (size_t)h->ps * h->ps);
    std::vector<int32_t> of(h->objFirst), oc(h->objCount);
    void* v;
    if (!r) { r = upload(h, &v, win); h->dWin = (double*)v; }
    if (!r) { r = upload(h, &v, nwin); h->dNWin = (double*)v; }
    if (!r) { r = upload(h, &v, h->imgObj); h->dImgObj = (int32_t*)v; }
    if (!r) { r = upload(h, &v, h->imgCh); h->dImgCh = (int32_t*)v; }
    if (!r) { r = upload(h, &v, of); h->dObjFirst = (int32_t*)v; }
    if (!r) { r = upload(h, &v, oc); h->dObjCount = (int32_t*)v; }
    if (!r) { r = upload(h, &v, h->objWeight); h->dObjW = (double*)v; }
    if (!r) { r = upload(h, &v, h->gradStep); h->dGradStep = (double*)v; }
    if (!r) {
        cudaError_t se = cudaSuccess;
        with_size(h->N, h->fp64, [&](auto L, auto) { se = decltype(L)::setup(h->M); });
        if (se != cudaSuccess) { h->err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(se); r = RDXG_ERR_CUDA; }
    }
    h->dObjFirstC = h->dObjFirst;
    h->dObjCountC = h->dObjCount;
    if (!r) {
        cudaError_t de = cudaDeviceGetAttribute(&h->numSMs, cudaDevAttrMultiProcessorCount, g->device);
        if (de != cudaSuccess) { h->err = cudaGetErrorString(de); r = RDXG_ERR_CUDA; }
        h->adjGrid = h->numSMs * 8;
        h->fdGrid = h->numSMs * 8;
    }
    if (!r) {
        // sizes whose work tile does not fit shared memory (FP64 at N = 128): one global tile
        // per block of the transform kernels, which run one image per block (at most the
        // batch's images; the finite-difference kernel strides over its items)
        const size_t cxs = h->fp64 ? 16 : 8, elems = (size_t)h->N * (h->N + 1);   // Tile<N>::ELEMS
        if ((elems + h->N) * cxs > kMaxSmem) {                                       // GlobalTile<T, N>
            h->gtileBlocks = h->Pmax * h->I;
            r = dalloc(h, &h->dGtile, (size_t)h->gtileBlocks * elems * cxs);
        }
    }
    const char* at = getenv("RDXG_AUTOTUNE");
    if (at && atoi(at) == 0) h->tune = 0;   // default shapes, no measurement
    const char* nf = getenv("RDXG_NO_FUSED");
    if (!r && !(nf && atoi(nf))) r = setup_fused(h, s);
    if (!r) r = upload_geometry(h);   // every patch shape 0 (the handle's own geometry)
    if (!r && !h->fused && !h->fp64) {
        // the general FP32 path (OTF size 128, or a support the half-plane evaluation does not
        // take): the mode expansion on the tensor cores ahead of the transform kernel
        const size_t G = (size_t)h->Pmax * h->I;
        r = dalloc(h, &h->dPhiImg, G * (size_t)h->n * h->n * sizeof(float));
        const char* pm = getenv("RDXG_PHASE_PARTS");
        const int parts = pm ? atoi(pm) : 3;
        if (!r) r = setup_phase_tc(h, parts == 0 || parts == 2 ? parts : 3);
    }
    if (!r && h->fused) {
        // rdxg_metric_noalloc's static scratch: its address in this context, which also loads
        // (and so reserves) it now rather than in that call
        cudaError_t ne = noalloc_scratch(&h->dNoAlloc);
        if (ne != cudaSuccess) { h->err = std::string("static scratch: ") + cudaGetErrorString(ne); r = RDXG_ERR_CUDA; }
    }
    if (!r) {
        // Kept or recomputed transforms: recomputed when keeping X, PF (and on the fused path S)
        // for every image would exceed the memory budget -- the device's free memory, or
        // RDXG_MEMORY_BUDGET bytes for the whole handle; RDXG_RECOMPUTE=0/1 forces the choice.
        with_size(h->N, h->fp64, [&](auto L, auto) { h->slotsPerSM = decltype(L)::recompute_occupancy(h->M); });
        int32_t* dq = nullptr;
        if ((r = dalloc_t(h, &dq, 1))) { *out = h; return r; }
        const cudaError_t qe = query_nsmid(dq, &h->nsmid, h->stream);
        dfree(h, &dq, sizeof(int32_t));
        if (qe != cudaSuccess) { h->err = std::string("SM count: ") + cudaGetErrorString(qe); *out = h; return RDXG_ERR_CUDA; }
        if (h->nsmid < h->numSMs) h->nsmid = h->numSMs;
        // the persistent recomputing kernels (block = slot) run one wave of resident blocks
        h->scrBlocks = h->slotsPerSM > 0 ? h->numSMs * h->slotsPerSM : 0;
        const size_t G = (size_t)h->Pmax * h->I, cxs = h->fp64 ? 16 : 8;
        const size_t S = h->fused ? 0 : G * (size_t)h->N * h->N * cxs;   // kept in both modes
        const size_t keep = kept_transform_bytes(h), scr = recompute_scratch_bytes(h);
        const char* mb = getenv("RDXG_MEMORY_BUDGET");
        const char* rcEnv = getenv("RDXG_RECOMPUTE");
        size_t budget = 0, freeB = 0, totalB = 0;
        if (mb) budget = (size_t)strtoull(mb, nullptr, 10);
        else if (cudaMemGetInfo(&freeB, &totalB) == cudaSuccess) budget = h->allocBytes + freeB;
        bool want = budget > 0 && h->allocBytes + S + keep + ((size_t)64 << 20) > budget;
        if (rcEnv) want = atoi(rcEnv) != 0;
        if (want && h->scrBlocks > 0 && budget > 0 && h->allocBytes + S + scr > budget) {
            char msg[256];
            std::snprintf(msg, sizeof(msg), "the batch needs %zu bytes even with recomputed transforms; the budget is "
                          "%zu bytes: fewer patches per handle", h->allocBytes + S + scr, budget);
            h->err = msg;
            r = RDXG_ERR_NOMEM;
        } else {
            r = setup_transforms(h, want && h->scrBlocks > 0);
        }
    }
    // RDXG_SHAPES="eval,forward,adjoint" (threads per block, 0 = default) pins the launch
    // shapes, e.g. for profiling runs, where the planner's timing would be distorted
    const char* shp = getenv("RDXG_SHAPES");
    if (!r && shp) {
        rdxg_launch_shape ls{};
        if (sscanf(shp, "%d,%d,%d", &ls.eval_threads, &ls.forward_threads, &ls.adjoint_threads) == 3) {
            if (ls.eval_threads && !h->fused) ls.eval_threads = 0;
            if (ls.forward_threads && h->fused) ls.forward_threads = 0;
            r = rdxg_set_launch_shape(h, &ls);
        }
    }
    *out = h;
    return r;
}

int rdxg_destroy(rdxg_solver* h) {
    if (!h) return RDXG_OK;
    for (void* p : h->allocs) cudaFree(p);
    if (h->hActive) cudaFreeHost(h->hActive);
    if (h->own) cudaStreamDestroy(h->own);
    if (h->side) cudaStreamDestroy(h->side);
    delete h;
    return RDXG_OK;
}

int rdxg_set_fit_plane(rdxg_solver* h, int32_t enable) {
    if (!h) return RDXG_ERR_ARG;
    if (enable && !h->dPlane) {
        const int r = dalloc_t(h, &h->dPlane, (size_t)h->Pmax * h->nObj * 2);
        if (r) return r;
    }
    h->fitPlane = enable != 0;
    // loaded patches are prepared again with (or without) the planes
    return h->loaded ? prepare_patches(h) : RDXG_OK;
}

int rdxg_set_reg_alpha(rdxg_solver* h, const double* weights) {
    if (!h) return RDXG_ERR_ARG;
    if (!weights) {
        h->hRegW.clear();
        return RDXG_OK;
    }
    if (!h->dRegW) {
        const int r = dalloc_t(h, &h->dRegW, (size_t)h->nPar);
        if (r) return r;
    }
    if (h->ragged) {
        h->err = "REG_ALPHA weights are per handle geometry; a ragged batch (rdxg_set_patch_shapes) does not take them";
        return RDXG_ERR_UNSUPPORTED;
    }
    h->hRegW.assign(weights, weights + h->nPar);
    // on the handle's stream, after any of its work still in flight
    CK(h, cudaMemcpyAsync(h->dRegW, h->hRegW.data(), (size_t)h->nPar * sizeof(double), cudaMemcpyHostToDevice,
                          h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return RDXG_OK;
}

extern "C++" {
namespace {
int set_start(rdxg_solver* h, const double* alpha, bool recut) {
    if (!h) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    if (alpha) {
        if (!h->dInitAlpha) {
            const int r = dalloc_t(h, &h->dInitAlpha, (size_t)h->Pmax * h->nPar);
            if (r) return r;
        }
        if (h->ragged) {
            // the image slots and modes a patch does not use start (and stay) at zero
            std::vector<double> a(alpha, alpha + (size_t)h->P * h->nPar);
            for (int p = 0; p < h->P; ++p) {
                const rdxg_solver::Shape& sh = h->shapes[h->patchShape[p]];
                for (int i = 0; i < h->nPar; ++i)
                    if (i / h->M >= sh.nImg || i % h->M >= sh.M) a[(size_t)p * h->nPar + i] = 0.0;
            }
            CK(h, cudaMemcpyAsync(h->dInitAlpha, a.data(), a.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  h->stream));
            CK(h, cudaStreamSynchronize(h->stream));
        } else {
            CK(h, cudaMemcpyAsync(h->dInitAlpha, alpha, (size_t)h->P * h->nPar * sizeof(double),
                                  cudaMemcpyHostToDevice, h->stream));
        }
    }
    h->haveInit = alpha != nullptr;
    h->initRecut = recut;
    return prepare_patches(h);
}
}  // namespace
}  // extern "C++"

int rdxg_set_initial_alpha(rdxg_solver* h, const double* alpha) { return set_start(h, alpha, true); }

int rdxg_set_patch_shapes(rdxg_solver* h, int32_t n_shapes, const rdxg_patch_shape* shapes, int32_t n_patches,
                          const int32_t* patch_shape) {
    if (!h) return RDXG_ERR_ARG;
    if (n_shapes <= 0) {
        // back to a uniform batch: every patch the handle's geometry
        h->shapes.resize(1);
        h->patchShape.assign(h->Pmax, 0);
        h->ragged = false;
        h->raggedPatches = 0;
        h->loaded = false;
        return upload_geometry(h);
    }
    if (!shapes || !patch_shape || n_patches < 1 || n_patches > h->Pmax) { h->err = "bad patch shapes"; return RDXG_ERR_ARG; }
    if (!h->hRegW.empty()) {
        h->err = "REG_ALPHA weights are per handle geometry; a ragged batch does not take them";
        return RDXG_ERR_UNSUPPORTED;
    }
    // every channel must have the same number of image slots (frames)
    std::vector<int> perCh(h->C, 0);
    for (int j = 0; j < h->I; ++j) perCh[h->imgCh[j]]++;
    const int F = perCh[0];
    for (int c = 0; c < h->C; ++c)
        if (perCh[c] != F) { h->err = "ragged batches need the same number of frames in every channel"; return RDXG_ERR_ARG; }
    const int needModes = std::max(h->geo.tilt_x, h->geo.tilt_y) + 1;
    std::vector<rdxg_solver::Shape> add(n_shapes);
    for (int k = 0; k < n_shapes; ++k) {
        const rdxg_patch_shape& ps = shapes[k];
        if (ps.frames < 1 || ps.frames > F || ps.n_modes < std::max(1, needModes) || ps.n_modes > h->M ||
            ps.n_free < 1 || ps.n_free > h->nFree || ps.ns_nnz < 0 || (ps.ns_nnz > 0 && (!ps.ns_rows || !ps.ns_cols || !ps.ns_vals))) {
            h->err = "patch shape " + std::to_string(k) + ": frames 1.." + std::to_string(F) + ", modes " +
                     std::to_string(std::max(1, needModes)) + ".." + std::to_string(h->M) + ", n_free 1.." +
                     std::to_string(h->nFree);
            return RDXG_ERR_ARG;
        }
        rdxg_solver::Shape& sh = add[k];
        sh.frames = ps.frames; sh.M = ps.n_modes; sh.nFree = ps.n_free;
        int r = shape_tables(h, sh);
        if (!r) r = shape_maps(h, sh, ps.ns_nnz, ps.ns_rows, ps.ns_cols, ps.ns_vals);
        if (r) return r;
    }
    for (int p = 0; p < n_patches; ++p)
        if (patch_shape[p] < 0 || patch_shape[p] >= n_shapes) { h->err = "patch_shape out of range"; return RDXG_ERR_ARG; }
    h->shapes.resize(1);
    h->shapes.insert(h->shapes.end(), add.begin(), add.end());
    h->patchShape.assign(h->Pmax, 0);
    for (int p = 0; p < n_patches; ++p) h->patchShape[p] = patch_shape[p] + 1;
    h->ragged = true;
    h->raggedPatches = n_patches;
    h->loaded = false;   // the next rdxg_set_patches loads the batch these shapes describe
    return upload_geometry(h);
}

int rdxg_set_start_alpha(rdxg_solver* h, const double* alpha) { return set_start(h, alpha, false); }

int rdxg_set_stream(rdxg_solver* h, void* st) {
    if (!h) return RDXG_ERR_ARG;
    h->stream = st ? (cudaStream_t)st : h->own;
    return RDXG_OK;
}

int rdxg_set_patches(rdxg_solver* h, int32_t P, const float* cut, const double* ra, const double* fg) {
    if (!h || !cut) return RDXG_ERR_ARG;
    if (P < 1 || P > h->Pmax) { h->err = "n_patches out of range"; return RDXG_ERR_ARG; }
    h->dCutExt = nullptr;
    CK(h, cudaMemcpyAsync(h->dCut, cut, (size_t)P * h->I * h->cs * h->cs * sizeof(float), cudaMemcpyHostToDevice, h->stream));
    return set_patches_common(h, P, ra, fg);
}

int rdxg_set_patches_device(rdxg_solver* h, int32_t P, const float* dcut, const double* ra, const double* fg) {
    if (!h || !dcut) return RDXG_ERR_ARG;
    h->dCutExt = dcut;
    return set_patches_common(h, P, ra, fg);
}

// REG_ALPHA on the host paths: Solver::metric adds 0.5 sum alpha^2 w (solver.cpp:804-811);
// Solver::gradient starts from alpha * w and assigns the data term to the enabled modes, so
// only the modes not enabled keep alpha * w (solver.cpp:860-885).
void add_reg_metric(const rdxg_solver* h, const double* alpha, double* metric) {
    if (h->hRegW.empty()) return;
    for (int p = 0; p < h->P; ++p) {
        double sum = 0;
        const double* a = alpha + (size_t)p * h->nPar;
        for (int i = 0; i < h->nPar; ++i) sum += 0.5 * a[i] * a[i] * h->hRegW[i];
        metric[p] += sum;
    }
}
void add_reg_gradient(const rdxg_solver* h, const double* alpha, const uint8_t* enabled, double* grad) {
    if (h->hRegW.empty() || !enabled) return;
    for (int p = 0; p < h->P; ++p)
        for (int i = 0; i < h->nPar; ++i)
            if (!enabled[i % h->M]) {
                const size_t k = (size_t)p * h->nPar + i;
                grad[k] = alpha[k] * h->hRegW[i];
            }
}

int rdxg_metric(rdxg_solver* h, const double* alpha, double* metric) {
    if (!h || !alpha || !metric) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    int r = h->fp64 ? upload_alpha<double>(h, alpha) : upload_alpha<float>(h, alpha);
    if (r) return r;
    if ((r = set_requests(h, REQ_F, GM_VOGEL, h->M)) || (r = reset_reference(h))) return r;
    if (h->fused) {
        // a first pass sets the reference object to this point, the second evaluates
        if ((r = fused_pass(h, REQ_F, 2))) return r;
        if ((r = fused_pass(h, REQ_F, 0))) return r;
        if ((r = metric_from_objects(h, metric))) return r;
        add_reg_metric(h, alpha, metric);
        return tc_check(h);
    }
    with_size(h->N, h->fp64, [&](auto L, auto t) {
        using T = decltype(t);
        KParams<T> kp = make_kparams<T>(h);
        phase_general(h, h->stream);
        decltype(L)::forward(kp, h->P * h->I, h->stream);
        launch_accum<T>(kp, h->P * h->nObj, h->stream);
    });
    CKL(h);
    if ((r = metric_from_partials(h, metric))) return r;
    add_reg_metric(h, alpha, metric);
    return RDXG_OK;
}

int rdxg_metric_noalloc(rdxg_solver* h, const double* alpha, double* metric) {
    if (!h || !alpha || !metric) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    if (!h->fused) {
        h->err = "rdxg_metric_noalloc: needs the FP32 half-plane evaluation (OTF size 32, 64 or 88 with a "
                 "symmetric OTF support)";
        return RDXG_ERR_UNSUPPORTED;
    }
    if (h->ragged) {
        h->err = "rdxg_metric_noalloc: takes uniform batches only (no rdxg_set_patch_shapes)";
        return RDXG_ERR_UNSUPPORTED;
    }
    int dev = -1;
    CK(h, cudaGetDevice(&dev));
    if (dev != h->geo.device) {
        h->err = "rdxg_metric_noalloc: the handle's device must be the current device";
        return RDXG_ERR_STATE;
    }
    void* base = h->dNoAlloc;
    if (!base) { h->err = "rdxg_metric_noalloc: the static scratch was not found"; return RDXG_ERR_STATE; }
    // carve the scratch into 256-byte aligned sections
    const size_t P = (size_t)h->P, G = P * h->I, PO = P * h->nObj, M = (size_t)h->M, n2 = (size_t)h->n * h->n;
    const size_t nH = (size_t)h->nH, cpp = (size_t)h->chunksPerPatch;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off += (bytes + 255) & ~(size_t)255;
        return o;
    };
    const size_t oAlpha = take(G * M * sizeof(double)), oAe = take(G * M * sizeof(float));
    const size_t oPhi = take(G * n2 * sizeof(float)), oPart = take(P * cpp * 4 * nH * sizeof(float));
    const size_t oObj = take(PO * h->nTilesH * sizeof(double)), oEval = take(P * cpp * sizeof(EvalItem));
    const size_t oPo = take(PO * sizeof(PoItem)), oEvalP = take(P * sizeof(int32_t));
    const size_t oCnt = take(kNumCounters * sizeof(int32_t)), oMetric = take(P * sizeof(double));
    if (off > kNoAllocScratchBytes) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "rdxg_metric_noalloc: %zu patches need %zu bytes of scratch; the static scratch holds %zu "
                      "bytes (at most %zu patches of this geometry)",
                      P, off, kNoAllocScratchBytes, kNoAllocScratchBytes / ((off + P - 1) / P));
        h->err = msg;
        return RDXG_ERR_UNSUPPORTED;
    }
    unsigned char* sb = static_cast<unsigned char*>(base);
    double* dAlpha = reinterpret_cast<double*>(sb + oAlpha);
    float* dAe = reinterpret_cast<float*>(sb + oAe);
    int32_t* cnt = reinterpret_cast<int32_t*>(sb + oCnt);
    double* dObj = reinterpret_cast<double*>(sb + oObj);
    double* dMetric = reinterpret_cast<double*>(sb + oMetric);
    Lists L{};
    L.eval = reinterpret_cast<EvalItem*>(sb + oEval);
    L.po = reinterpret_cast<PoItem*>(sb + oPo);
    L.evalP = reinterpret_cast<int32_t*>(sb + oEvalP);
    L.counters = cnt;
    L.nEval = cnt + 0; L.nPo = cnt + 1; L.nGradP = cnt + 2; L.nFdP = cnt + 3; L.nEvalP = cnt + 4;
    CK(h, cudaMemcpyAsync(dAlpha, alpha, G * M * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    // the list counters start at zero; every other word read below is written first
    CK(h, cudaMemsetAsync(cnt, 0, kNumCounters * sizeof(int32_t), h->stream));
    launch_noalloc_alpha(dAlpha, h->dCurTilt, h->dResAlpha, (int)G, (int)M, h->geo.tilt_x, h->geo.tilt_y, dAe,
                         h->stream);
    // as rdxg_metric: a first pass sets the reference object to this point, the second evaluates
    for (int mode : {2, 0}) {
        launch_noalloc_lists(h->P, h->nObj, h->dObjFirst, h->dObjCount, h->dObjChunk0, h->chunk, h->chunksPerPatch,
                             mode, L, h->stream);
        with_eval(h->N, [&](auto E) {
            EvalParams<float> e = make_evalparams<float>(h);
            e.k.alphaEff = dAe;
            e.phi = reinterpret_cast<float*>(sb + oPhi);
            e.part = reinterpret_cast<Acc4<float>*>(sb + oPart);
            e.objMetric = dObj;
            e.L = L;
            decltype(E)::phase(e, h->phaseGrid, h->stream);
            decltype(E)::eval(e, h->npt, h->evalGrid, h->stream);
            decltype(E)::reduce(e, h->reduceGrid, h->stream);
        });
    }
    launch_noalloc_metric(dObj, h->P, h->nObj, h->nTilesH, h->dObjW, (double)h->ps * h->ps, dMetric, h->stream);
    CKL(h);
    CK(h, cudaMemcpyAsync(metric, dMetric, P * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    add_reg_metric(h, alpha, metric);
    return tc_check(h);
}

int rdxg_metric_with_reference(rdxg_solver* h, const double* alpha_ref, const double* alpha, double* metric) {
    if (!h || !alpha_ref || !alpha || !metric) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    if (!h->fused) return rdxg_metric(h, alpha, metric);
    int r;
    if ((r = upload_alpha<float>(h, alpha_ref)) || (r = set_requests(h, REQ_F, GM_VOGEL, h->M)) ||
        (r = reset_reference(h)) || (r = fused_pass(h, REQ_F, 2)))
        return r;
    if ((r = upload_alpha<float>(h, alpha)) || (r = fused_pass(h, REQ_F, 0))) return r;
    if ((r = metric_from_objects(h, metric))) return r;
    add_reg_metric(h, alpha, metric);
    return tc_check(h);
}

int rdxg_restore(rdxg_solver* h, const double* alpha, const double* frequency_cutoff, int32_t no_filter,
                 float* objects) {
    return rdxg_restore_ex(h, alpha, frequency_cutoff, no_filter, 0, objects, nullptr, nullptr, nullptr);
}

extern "C++" {
namespace {
int restore_impl(rdxg_solver* h, const double* alpha, const double* frequency_cutoff, int32_t no_filter,
                 int32_t outputs, float* objects, float* psf, float* cobj, float* res);
}  // namespace
}  // extern "C++"

int rdxg_restore_ex(rdxg_solver* h, const double* alpha, const double* frequency_cutoff, int32_t no_filter,
                    int32_t outputs, float* objects, float* psf, float* cobj, float* res) {
    if (!h) return RDXG_ERR_ARG;
    // with recomputed transforms the fused path keeps no OTFs: the restoration holds them for
    // the call
    const size_t sBytes = (size_t)h->Pmax * h->I * h->N * h->N * sizeof(float2);
    const bool tmpS = h->fused && !h->dS;
    if (tmpS) {
        const int r = dalloc(h, &h->dS, sBytes);
        if (r) return r;
    }
    const int r = restore_impl(h, alpha, frequency_cutoff, no_filter, outputs, objects, psf, cobj, res);
    if (tmpS) {
        cudaStreamSynchronize(h->stream);
        dfree(h, &h->dS, sBytes);
    }
    return r;
}

extern "C++" {
namespace {
int restore_impl(rdxg_solver* h, const double* alpha, const double* frequency_cutoff, int32_t no_filter,
                 int32_t outputs, float* objects, float* psf, float* cobj, float* res) {
    if (!h || !alpha || !frequency_cutoff || !objects) return RDXG_ERR_ARG;
    if (outputs & ~(RDXG_RESTORE_PSF | RDXG_RESTORE_PSF_AVG | RDXG_RESTORE_COBJ | RDXG_RESTORE_RESIDUAL))
        return RDXG_ERR_ARG;
    if ((outputs & (RDXG_RESTORE_PSF | RDXG_RESTORE_PSF_AVG)) && !psf) return RDXG_ERR_ARG;
    if ((outputs & RDXG_RESTORE_COBJ) && !cobj) return RDXG_ERR_ARG;
    if ((outputs & RDXG_RESTORE_RESIDUAL) && !res) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    // the mean PSF takes precedence over the per-image PSFs (object.cpp:337)
    if (outputs & RDXG_RESTORE_PSF_AVG) outputs &= ~RDXG_RESTORE_PSF;
    int r = h->fp64 ? upload_alpha<double>(h, alpha) : upload_alpha<float>(h, alpha);
    if (r) return r;
    // the OTFs at alpha on the full plane: a gradient-type evaluation keeps them
    if ((r = set_requests(h, REQ_DF, GM_VOGEL, h->M)) || (r = reset_reference(h))) return r;
    if (h->fused) {
        if ((r = fused_pass(h, REQ_DF, 1))) return r;
    } else {
        with_size(h->N, h->fp64, [&](auto L, auto t) {
            using T = decltype(t);
            KParams<T> kp = make_kparams<T>(h);
            phase_general(h, h->stream);
            decltype(L)::forward(kp, h->P * h->I, h->stream);
        });
    }
    const size_t N2 = (size_t)h->N * h->N;
    if (!h->dRestore) {
        if ((r = dalloc_t(h, &h->dRestore, (size_t)h->Pmax * h->nObj * kRestoreScratch * N2)) ||
            (r = dalloc_t(h, &h->dFc, (size_t)h->nObj)))
            return r;
    }
    CK(h, cudaMemcpyAsync(h->dFc, frequency_cutoff, h->nObj * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    if (!h->dRestoreOut && (r = dalloc_t(h, &h->dRestoreOut, (size_t)h->Pmax * h->nObj * h->ps * h->ps))) return r;
    const size_t PO = (size_t)h->Pmax * h->nObj, G = (size_t)h->Pmax * h->I, ps2 = (size_t)h->ps * h->ps;
    const int outGrid = h->numSMs * 2;
    if (outputs && !h->dObjFull) {
        if ((r = dalloc_t(h, &h->dObjFull, PO * N2)) || (r = dalloc(h, (void**)&h->dFo, PO * N2 * 2 * sizeof(double))) ||
            (r = dalloc_t(h, &h->dOutPool, (size_t)outGrid * 3 * N2)) || (r = dalloc_t(h, &h->dPsf, G * ps2)) ||
            (r = dalloc_t(h, &h->dCobj, G * ps2)) || (r = dalloc_t(h, &h->dRes, G * ps2)))
            return r;
    }
    RestoreArgs ra{h->dFc, no_filter ? 1 : 0, h->dRestore, h->dRestoreOut, outputs ? h->dObjFull : nullptr};
    RestoreOutArgs oa{outputs, h->dObjFull, (cx<double>*)h->dFo, h->dOutPool, h->dPsf, h->dCobj, h->dRes};
    cudaError_t ce = cudaSuccess;
    with_size(h->N, h->fp64, [&](auto L, auto t) {
        using T = decltype(t);
        KParams<T> kp = make_kparams<T>(h);
        ce = decltype(L)::restore(kp, ra, h->P * h->nObj, h->stream);
        if (ce == cudaSuccess && outputs) ce = decltype(L)::restore_outputs(kp, oa, outGrid, h->stream);
    });
    if (ce != cudaSuccess) { h->err = std::string("restore: ") + cudaGetErrorString(ce); return RDXG_ERR_CUDA; }
    if (h->fitPlane) {   // after the convolved objects and residuals, as the reference
        launch_add_plane(h->dPlane, h->dRestoreOut, h->P * h->nObj, h->ps, h->stream);
        CKL(h);
    }
    const size_t P = h->P;
    CK(h, cudaMemcpyAsync(objects, h->dRestoreOut, P * h->nObj * ps2 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    if (outputs & RDXG_RESTORE_PSF_AVG)
        CK(h, cudaMemcpyAsync(psf, h->dPsf, P * h->nObj * ps2 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    if (outputs & RDXG_RESTORE_PSF)
        CK(h, cudaMemcpyAsync(psf, h->dPsf, P * h->I * ps2 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    if (outputs & RDXG_RESTORE_COBJ)
        CK(h, cudaMemcpyAsync(cobj, h->dCobj, P * h->I * ps2 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    if (outputs & RDXG_RESTORE_RESIDUAL)
        CK(h, cudaMemcpyAsync(res, h->dRes, P * h->I * ps2 * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    return RDXG_OK;
}
}  // namespace
}  // extern "C++"

int rdxg_gradient(rdxg_solver* h, const double* alpha, const uint8_t* enabled, int32_t method, double* grad,
                  double* metric) {
    if (!h || !alpha || !grad) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    if (method != RDXG_GRAD_VOGEL && method != RDXG_GRAD_EXACT && method != RDXG_GRAD_FD) return RDXG_ERR_ARG;
    int r = h->fp64 ? upload_alpha<double>(h, alpha) : upload_alpha<float>(h, alpha);
    if (r) return r;
    const int gm = method == RDXG_GRAD_FD ? GM_FD : GM_VOGEL;
    if ((r = set_requests(h, REQ_DF, gm, h->M)) || (r = reset_reference(h))) return r;
    if (h->fused) {
        if ((r = fused_pass(h, REQ_DF, 1))) return r;
    }
    with_size(h->N, h->fp64, [&](auto L, auto t) {
        using T = decltype(t);
        KParams<T> kp = make_kparams<T>(h);
        if (!h->fused) {
            phase_general(h, h->stream);
            decltype(L)::forward(kp, h->P * h->I, h->stream);
            launch_accum<T>(kp, h->P * h->nObj, h->stream);
        }
        if (method != RDXG_GRAD_FD)
            decltype(L)::adjoint(kp, h->adjGrid, method == RDXG_GRAD_EXACT ? GK_EXACT : GK_VOGEL, h->stream);
    });
    if (method == RDXG_GRAD_FD) launch_fd(h);
    CKL(h);
    const size_t G = (size_t)h->P * h->I;
    CK(h, cudaMemcpyAsync(grad, h->dGalpha, G * h->M * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    if ((r = tc_check(h))) return r;
    if (enabled)
        for (size_t g = 0; g < G; ++g)
            for (int m = 0; m < h->M; ++m)
                if (!enabled[m]) grad[g * h->M + m] = 0.0;
    add_reg_gradient(h, alpha, enabled, grad);
    if (metric) {
        if (h->fused) {
            // the gradient pass left the exact object of this point as the reference
            if ((r = set_requests(h, REQ_F, GM_VOGEL, h->M)) || (r = fused_pass(h, REQ_F, 0))) return r;
            if ((r = metric_from_objects(h, metric))) return r;
        } else if ((r = metric_from_partials(h, metric))) {
            return r;
        }
        add_reg_metric(h, alpha, metric);
    }
    return RDXG_OK;
}

extern "C++" {
namespace {

// What a solve of one handle needs once its state is reset: the solver kernel's parameters
// and the re-shifts' arguments.
struct SolvePlan {
    rdxg_solver* h = nullptr;
    CgParams prm{};
    ShiftArgs sa{};
};

int plan_shapes_once(rdxg_solver* h);   // the launch-shape planner (below)

// Everything rdxg_solve_async does before the rounds: state reset on the handle's stream.
int prepare_solve(rdxg_solver* h, const rdxg_solve_params* s, SolvePlan& pl) {
    if (!h || !s) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    int r;
    if ((r = plan_shapes_once(h))) return r;
    if (h->dirty && (r = prepare_patches(h))) return r;
    h->dirty = true;
    h->launches = 0;
    h->lastParams = *s;
    pl.h = h;
    pl.prm = make_cg_params(h, s);
    if (pl.prm.max_metrics != h->maxMetrics) {
        if (h->dMetrics) {
            for (auto it = h->allocs.begin(); it != h->allocs.end(); ++it)
                if (*it == h->dMetrics) { cudaFree(*it); h->allocs.erase(it); break; }
            h->dMetrics = nullptr;
        }
        if ((r = dalloc_t(h, &h->dMetrics, (size_t)h->Pmax * pl.prm.max_metrics))) return r;
        h->maxMetrics = pl.prm.max_metrics;
    }
    const int P = h->P;
    CK(h, cudaMemsetAsync(h->dStates, 0, P * sizeof(CgState), h->stream));
    CK(h, cudaMemsetAsync(h->dVec, 0, (size_t)P * 5 * h->nFree * sizeof(double), h->stream));
    CK(h, cudaMemsetAsync(h->dAlphaOff, 0, (size_t)P * h->nPar * sizeof(double), h->stream));
    CK(h, cudaMemsetAsync(h->dAlpha, 0, (size_t)P * h->nPar * sizeof(double), h->stream));
    if (h->fused) {
        CK(h, cudaMemsetAsync(h->dOh, 0, (size_t)P * h->nObj * h->nH * sizeof(float2), h->stream));
        CK(h, cudaMemsetAsync(h->dAux, 0, (size_t)P * 2 * sizeof(int32_t), h->stream));
    }
    if (h->haveInit)   // alpha_offset = the initial coefficients
        CK(h, cudaMemcpyAsync(h->dAlphaOff, h->dInitAlpha, (size_t)P * h->nPar * sizeof(double),
                              cudaMemcpyDeviceToDevice, h->stream));
    launch_to_float(h->dAlphaOff, h->dAlphaOffF, (size_t)P * h->nPar, h->stream);
    CKL(h);
    pl.sa = make_shift_args(h);
    // the solver kernel stages its patch's data in shared memory when it fits
    size_t bytes = 0;
    cg_stage_choice(h, &h->cgStage, &h->cgStageMap, &bytes);
    if (h->cgStage) CK(h, h->fp64 ? setup_cg<double>(bytes) : setup_cg<float>(bytes));
    return RDXG_OK;
}

// One round of one handle on stream st: the solver kernel (with the re-shifts),
// [re-initialisation], evaluation, [adjoint], [finite differences]; optional(k, issue) issues
// the bracketed kernels.
template <typename Opt>
int issue_round(const SolvePlan& pl, cudaStream_t st, const ShiftArgs& sar, Opt&& optional) {
    rdxg_solver* h = pl.h;
    if (cudaMemsetAsync(h->dActive, 0, sizeof(int32_t), st) != cudaSuccess ||
        cudaMemsetAsync(h->dCounters, 0, kNumCounters * sizeof(int32_t), st) != cudaSuccess)
        return 1;
    const int P = h->P, G = P * h->I;
    with_size(h->N, h->fp64, [&](auto L, auto t) {
        using T = decltype(t);
        KParams<T> kp = make_kparams<T>(h);
        CgArgs<T> ca = make_cgargs<T>(h, pl.prm);
        launch_cg<T>(ca, sar, P, st);    // with the re-shifts of its patches
        optional(0, [&](cudaStream_t s2) {
            // Object::reInitialize: refit the planes of objects with shifted images, then
            // re-initialise their images
            if (h->fitPlane) launch_fit_plane<T>(kp, 0, P * h->nObj, s2);
            decltype(L)::prep(kp, 0, G, s2);
        });
        if (h->fused) {
            with_eval(h->N, [&](auto E) {
                EvalParams<float> e = make_evalparams<float>(h);
                decltype(E)::phase(e, h->phaseGrid, st);
                decltype(E)::eval(e, h->npt, h->evalGrid, st);
                decltype(E)::reduce(e, h->reduceGrid, st);
            });
        } else {
            phase_general(h, st);
            decltype(L)::forward(kp, G, st);
            launch_accum<T>(kp, P * h->nObj, st);
        }
        optional(1, [&](cudaStream_t s2) { decltype(L)::adjoint(kp, h->adjGrid, GK_VOGEL, s2); });
    });
    optional(2, [&](cudaStream_t s2) { launch_fd(h, s2); });
    return 0;
}

// Runs every plan's rounds as one CUDA graph, launched once per solve.  The graph is a WHILE
// node whose body holds `check` rounds of every handle -- one branch per handle, forked from
// the first handle's stream (handles sharing a stream are issued one after the other) and
// joined -- followed by k_loop_cond, which keeps the loop going while any handle has an active
// patch; the rounds run on the device with no host round trip.  The kernels that are only
// needed in some rounds (image re-initialisation after a re-shift, the adjoint, the
// finite-difference gradient) sit in IF nodes inside the body, whose conditions the last block
// of the round's solver kernel sets from the round's work-list counters.
int solve_rounds_graph(std::vector<SolvePlan>& plans, int check) {
    rdxg_solver* h0 = plans[0].h;
    cudaStream_t origin = h0->stream;
    const size_t nPlans = plans.size();
    for (SolvePlan& pl : plans) {
        rdxg_solver* h = pl.h;
        if (!h->side) CK(h, cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
        if (!h->dLaunchCount) {
            int r = dalloc_t(h, &h->dLaunchCount, 1);
            if (r) return r;
        }
        CK(h, cudaMemsetAsync(h->dLaunchCount, 0, sizeof(unsigned long long), h->stream));
        // the reset of every handle's state is complete before the graph runs on the origin
        if (h->stream != origin) CK(h, cudaStreamSynchronize(h->stream));
    }
    if (h0->activeListCap < (int)nPlans) {
        dfree(h0, &h0->dActiveList, (size_t)h0->activeListCap * sizeof(int32_t*));
        int r = dalloc_t(h0, &h0->dActiveList, nPlans);
        if (r) return r;
        h0->activeListCap = (int)nPlans;
    }
    if (!h0->dRounds) {
        int r = dalloc_t(h0, &h0->dRounds, 1);
        if (!r) r = dalloc_t(h0, &h0->dOverrun, 1);
        if (r) return r;
    }
    {
        std::vector<int32_t*> act(nPlans);
        for (size_t k = 0; k < nPlans; ++k) act[k] = plans[k].h->dActive;
        CK(h0, cudaMemcpyAsync(h0->dActiveList, act.data(), nPlans * sizeof(int32_t*), cudaMemcpyHostToDevice, origin));
        CK(h0, cudaMemsetAsync(h0->dRounds, 0, sizeof(long long), origin));
        CK(h0, cudaMemsetAsync(h0->dOverrun, 0, sizeof(int32_t), origin));
        CK(h0, cudaStreamSynchronize(origin));   // the host vector goes out of scope
    }
    std::vector<cudaEvent_t> ev(nPlans + 1, nullptr);
    cudaError_t ce = cudaSuccess;
    const char* what = "events";
    const auto tBuild = std::chrono::steady_clock::now();
    for (size_t k = 0; k <= nPlans && ce == cudaSuccess; ++k) ce = cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming);
    // the top-level graph: one WHILE node (its condition starts at 1 on every launch)
    cudaGraph_t top = nullptr, body = nullptr;
    cudaGraphConditionalHandle loop = 0;
    if (ce == cudaSuccess) { what = "graph"; ce = cudaGraphCreate(&top, 0); }
    if (ce == cudaSuccess) {
        what = "loop handle";
        ce = cudaGraphConditionalHandleCreate(&loop, top, 1, cudaGraphCondAssignDefault);
    }
    if (ce == cudaSuccess) {
        what = "loop node";
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = loop;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        if ((ce = cudaGraphAddNode(&node, top, nullptr, nullptr, 0, &np)) == cudaSuccess) body = np.conditional.phGraph_out[0];
    }
    bool capturing = false;
    if (ce == cudaSuccess) {
        what = "begin capture";
        ce = cudaStreamBeginCaptureToGraph(origin, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
        capturing = ce == cudaSuccess;
    }
    // fork: every other stream joins the capture after the origin's start
    if (ce == cudaSuccess && (ce = cudaEventRecord(ev[nPlans], origin)) == cudaSuccess) {
        for (size_t k = 0; k < nPlans && ce == cudaSuccess; ++k)
            if (plans[k].h->stream != origin) ce = cudaStreamWaitEvent(plans[k].h->stream, ev[nPlans], 0);
    }
    for (int r = 0; r < check && ce == cudaSuccess; ++r) {
        for (size_t k = 0; k < nPlans && ce == cudaSuccess; ++k) {
            SolvePlan& pl = plans[k];
            rdxg_solver* h = pl.h;
            cudaStream_t st = h->stream;
            // a conditional handle belongs to one conditional node: three new ones per round,
            // in the graph that holds the nodes (the loop's body)
            cudaGraphConditionalHandle cond[3] = {};
            what = "conditional handle";
            for (int c = 0; c < 3 && ce == cudaSuccess; ++c) ce = cudaGraphConditionalHandleCreate(&cond[c], body, 0, 0);
            if (ce != cudaSuccess) break;
            ShiftArgs sa = pl.sa;
            sa.useConditions = 1;
            sa.counters = h->dCounters;
            sa.fixedLaunches = (h->fused || h->tcPlan.valid) ? 4 : 3;
            sa.prepLaunches = h->fitPlane ? 2 : 1;
            sa.launchCount = h->dLaunchCount;
            sa.condPrep = cond[0];
            sa.condAdjoint = cond[1];
            sa.condFd = cond[2];
            // optional kernel c: an IF node on cond[c] after the stream's captured work so far,
            // its body captured on the handle's side stream
            auto optional = [&](int c, auto issue) {
                if (ce != cudaSuccess) return;
                cudaStreamCaptureStatus status;
                cudaGraph_t g = nullptr;
                const cudaGraphNode_t* deps = nullptr;
                size_t nDeps = 0;
                what = "capture info";
                if ((ce = cudaStreamGetCaptureInfo(st, &status, nullptr, &g, &deps, nullptr, &nDeps)) != cudaSuccess)
                    return;
                what = "conditional node";
                cudaGraphNodeParams np{};
                np.type = cudaGraphNodeTypeConditional;
                np.conditional.handle = cond[c];
                np.conditional.type = cudaGraphCondTypeIf;
                np.conditional.size = 1;
                cudaGraphNode_t node;
                if ((ce = cudaGraphAddNode(&node, g, deps, nullptr, nDeps, &np)) != cudaSuccess) return;
                what = "capture dependencies";
                if ((ce = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1,
                                                              cudaStreamSetCaptureDependencies)) != cudaSuccess)
                    return;
                what = "body capture";
                cudaGraph_t ib = np.conditional.phGraph_out[0];
                if ((ce = cudaStreamBeginCaptureToGraph(h->side, ib, nullptr, nullptr, 0,
                                                        cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
                    return;
                issue(h->side);
                ce = cudaStreamEndCapture(h->side, &ib);
            };
            if (issue_round(pl, st, sa, optional)) { ce = cudaErrorUnknown; what = "round"; }
            if (ce == cudaSuccess && (ce = cudaGetLastError()) != cudaSuccess) what = "kernel launch";
        }
    }
    // join: the origin waits for every branch, then decides whether the loop goes on
    for (size_t k = 0; k < nPlans && ce == cudaSuccess; ++k) {
        cudaStream_t st = plans[k].h->stream;
        if (st == origin) continue;
        what = "join";
        if ((ce = cudaEventRecord(ev[k], st)) == cudaSuccess) ce = cudaStreamWaitEvent(origin, ev[k], 0);
    }
    if (ce == cudaSuccess) {
        LoopArgs la;
        la.loop = loop;
        la.active = h0->dActiveList;
        la.nActive = (int32_t)nPlans;
        la.roundsPerIteration = check;
        // a round is one evaluation of every active patch, and a CG iteration takes one
        // gradient and a line search of a few to a few hundred metrics: far more rounds than
        // that means a state machine that stopped advancing
        long long maxIter = 0;
        for (const SolvePlan& pl : plans) maxIter = std::max<long long>(maxIter, pl.prm.max_iterations);
        la.maxRounds = std::min<long long>(2000000LL, 1000LL * maxIter + 10000LL);
        la.rounds = h0->dRounds;
        la.overrun = h0->dOverrun;
        la.launchCount = h0->dLaunchCount;
        launch_loop_cond(la, origin);
        if ((ce = cudaGetLastError()) != cudaSuccess) what = "loop condition";
    }
    if (capturing) {
        cudaGraph_t captured = body;
        const cudaError_t ee = cudaStreamEndCapture(origin, &captured);
        if (ce == cudaSuccess && ee != cudaSuccess) { ce = ee; what = "end capture"; }
    }
    cudaGraphExec_t exec = nullptr;
    if (ce == cudaSuccess && (ce = cudaGraphInstantiate(&exec, top, 0)) != cudaSuccess) what = "instantiate";
    int r = RDXG_OK;
    if (ce != cudaSuccess) {
        cudaGetLastError();
        h0->err = std::string("solver graph (") + what + "): " + cudaGetErrorString(ce);
        r = RDXG_ERR_CUDA;
    }
    const auto tRun = std::chrono::steady_clock::now();
    if (r == RDXG_OK) {
        int32_t overrun = 0;
        if ((ce = cudaGraphLaunch(exec, origin)) == cudaSuccess &&
            (ce = cudaMemcpyAsync(h0->hActive, h0->dOverrun, sizeof(int32_t), cudaMemcpyDeviceToHost, origin)) ==
                cudaSuccess &&
            (ce = cudaStreamSynchronize(origin)) == cudaSuccess) {
            overrun = *h0->hActive;
        }
        if (ce != cudaSuccess) {
            h0->err = std::string("solver graph launch: ") + cudaGetErrorString(ce);
            r = RDXG_ERR_CUDA;
        } else if (overrun) {
            h0->err = "solver did not terminate";
            r = RDXG_ERR_STATE;
        }
    }
    if (getenv("RDXG_VERBOSE")) {
        const auto tEnd = std::chrono::steady_clock::now();
        fprintf(stderr, "solve graph: built and instantiated in %.3f ms, ran in %.3f ms\n",
                std::chrono::duration<double, std::milli>(tRun - tBuild).count(),
                std::chrono::duration<double, std::milli>(tEnd - tRun).count());
    }
    if (exec) cudaGraphExecDestroy(exec);
    if (top) cudaGraphDestroy(top);
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
    if (r) return r;
    for (SolvePlan& pl : plans) {
        unsigned long long n = 0;
        CK(pl.h, cudaMemcpy(&n, pl.h->dLaunchCount, sizeof(n), cudaMemcpyDeviceToHost));
        pl.h->launches = (int64_t)n;
    }
    return RDXG_OK;
}

}  // namespace
}  // extern "C++"

// RDXG_NO_GRAPH=1: the rounds issued from a host loop, every kernel launched every round, each
// handle on its own stream (for profilers that do not take kernels out of graphs with
// conditional nodes); the host reads the active counters every `check` rounds.
static bool no_graph() {
    const char* ng = getenv("RDXG_NO_GRAPH");
    return ng && atoi(ng);
}

static int solve_rounds_host(std::vector<SolvePlan>& plans, int check) {
    for (long round = 0;; ++round) {
        for (const SolvePlan& pl : plans) {
            rdxg_solver* h = pl.h;
            if (issue_round(pl, h->stream, pl.sa, [&](int, auto issue) { issue(h->stream); })) {
                h->err = "cudaMemsetAsync failed";
                return RDXG_ERR_CUDA;
            }
            h->launches += (h->fused ? 7 : (h->tcPlan.valid ? 7 : 6)) + (h->fitPlane ? 1 : 0);
            CKL(h);
        }
        if ((round + 1) % check == 0) {
            int32_t active = 0;
            for (const SolvePlan& pl : plans) {
                rdxg_solver* h = pl.h;
                CK(h, cudaMemcpyAsync(h->hActive, h->dActive, sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
                CK(h, cudaStreamSynchronize(h->stream));
                active += *h->hActive;
            }
            if (active == 0) break;
        }
        if (round > 2000000L) { plans[0].h->err = "solver did not terminate"; return RDXG_ERR_STATE; }
    }
    return RDXG_OK;
}

int rdxg_solve_async(rdxg_solver* h, const rdxg_solve_params* s) {
    std::vector<SolvePlan> plans(1);
    int r = prepare_solve(h, s, plans[0]);
    if (r) return r;
    const int check = s->check_every > 0 ? s->check_every : 8;
    return no_graph() ? solve_rounds_host(plans, check) : solve_rounds_graph(plans, check);
}

int rdxg_solve_many(rdxg_solver* const* handles, int32_t n, const rdxg_solve_params* s) {
    if (!handles || n < 1 || !s) return RDXG_ERR_ARG;
    std::vector<SolvePlan> plans(n);
    for (int k = 0; k < n; ++k) {
        if (!handles[k]) return RDXG_ERR_ARG;
        for (int j = 0; j < k; ++j)
            if (handles[j] == handles[k]) { handles[k]->err = "a handle appears twice"; return RDXG_ERR_ARG; }
        if (handles[k]->geo.device != handles[0]->geo.device) {
            handles[k]->err = "handles on different devices";
            return RDXG_ERR_ARG;
        }
        const int r = prepare_solve(handles[k], s, plans[k]);
        if (r) return r;
    }
    const int check = s->check_every > 0 ? s->check_every : 8;
    return no_graph() ? solve_rounds_host(plans, check) : solve_rounds_graph(plans, check);
}

int rdxg_fetch_results(rdxg_solver* h, double* alpha_out, rdxg_patch_report* reports, double* metrics) {
    if (!h) return RDXG_ERR_ARG;
    const int P = h->P;
    if (alpha_out)
        CK(h, cudaMemcpyAsync(alpha_out, h->dAlpha, (size_t)P * h->nPar * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    std::vector<CgState> st(P);
    CK(h, cudaMemcpyAsync(st.data(), h->dStates, P * sizeof(CgState), cudaMemcpyDeviceToHost, h->stream));
    if (metrics && h->dMetrics)
        CK(h, cudaMemcpyAsync(metrics, h->dMetrics, (size_t)P * h->maxMetrics * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(h, cudaStreamSynchronize(h->stream));
    int r = tc_check(h);
    if (r) return r;
    if (reports) {
        for (int p = 0; p < P; ++p) {
            rdxg_patch_report& r = reports[p];
            r.initial_metric = st[p].initial_metric;
            r.final_metric = st[p].this_metric;
            r.iterations = st[p].total_iterations;
            r.status = st[p].status == ST_FAILURE ? 1 : 0;
            r.n_f_evals = st[p].n_f;
            r.n_df_evals = st[p].n_df;
            r.fail_count = st[p].fail_count;
            r.n_metrics = st[p].n_metrics;
        }
    }
    return RDXG_OK;
}

int rdxg_solve(rdxg_solver* h, const rdxg_solve_params* s, double* alpha_out, rdxg_patch_report* reports,
               double* metrics) {
    int r = rdxg_solve_async(h, s);
    if (r) return r;
    return rdxg_fetch_results(h, alpha_out, reports, metrics);
}

int64_t rdxg_last_launch_count(const rdxg_solver* h) { return h ? h->launches : 0; }

int rdxg_set_phase_mode(rdxg_solver* h, int32_t mode) {
    if (!h || (mode != 0 && mode != 2 && mode != 3)) return RDXG_ERR_ARG;
    if (h->fp64) {
        if (mode == 0) return RDXG_OK;
        h->err = "the general path in FP64 expands the modes inside its transform kernel (CUDA cores only)";
        return RDXG_ERR_STATE;
    }
    const int r = setup_phase_tc(h, mode);
    if (r) return r;
    if (mode != 0 && !h->tcPlan.valid) {
        h->err = "the tensor-core mode expansion does not take this shape";
        return RDXG_ERR_STATE;
    }
    return RDXG_OK;
}

int32_t rdxg_phase_mode(const rdxg_solver* h) {
    if (!h || h->fp64) return 0;
    return h->tcPlan.valid ? h->tcPlan.parts : 0;
}

int rdxg_set_recompute(rdxg_solver* h, int32_t on) {
    if (!h || (on != 0 && on != 1)) return RDXG_ERR_ARG;
    CK(h, cudaStreamSynchronize(h->stream));   // no kernel of the handle reads the buffers any more
    return setup_transforms(h, on != 0);
}

int32_t rdxg_recompute(const rdxg_solver* h) { return h && h->recompute ? 1 : 0; }

extern "C++" {
namespace {

// Times kernel `k` (0 forward of a metric evaluation, 1 per-object accumulation, 2 forward of
// a gradient evaluation, 3 analytic adjoint, 4 finite-difference gradient) on the loaded batch
// at its current point: average ms per launch over reps launches after one warm-up, with
// CUDA events on the handle's stream.  nGrad > 0: the adjoint works on the first nGrad
// patches only (the size of a solve round's gradient list).
int time_kernel(rdxg_solver* h, int k, int reps, cudaEvent_t e0, cudaEvent_t e1, double* ms, int nGrad = 0) {
    const int G = h->P * h->I, PO = h->P * h->nObj;
    const int req = (k < 2) ? REQ_F : REQ_DF;
    const int gm = (k == 4) ? GM_FD : GM_VOGEL;
    int r;
    if ((r = set_requests(h, req, gm, h->M))) return r;
    if (h->fused && (r = host_lists(h, req, req == REQ_DF ? 1 : 0))) return r;
    auto launch = [&](int which) {
        with_size(h->N, h->fp64, [&](auto L, auto t) {
            using T = decltype(t);
            KParams<T> kp = make_kparams<T>(h);
            if (h->fused && which <= 2) {
                with_eval(h->N, [&](auto E) {
                    EvalParams<float> e = make_evalparams<float>(h);
                    if (which == 1) {
                        decltype(E)::reduce(e, h->reduceGrid, h->stream);
                    } else {
                        decltype(E)::phase(e, h->phaseGrid, h->stream);
                        decltype(E)::eval(e, h->npt, h->evalGrid, h->stream);
                    }
                });
                return;
            }
            switch (which) {
                case 0: case 2: phase_general(h, h->stream); decltype(L)::forward(kp, G, h->stream); break;
                case 1: launch_accum<T>(kp, PO, h->stream); break;
                case 3: decltype(L)::adjoint(kp, h->adjGrid, GK_VOGEL, h->stream); break;
                case 4: launch_fd(h); break;
            }
        });
    };
    // inputs of the timed kernel: forward and accumulation in the requested mode
    if (k >= 3) { launch(2); launch(1); }
    if (k == 1) launch(0);
    if (k == 3 && nGrad > 0 && nGrad < h->P) {
        const int32_t n = nGrad;
        CK(h, cudaMemcpyAsync(h->dCounters + 2, &n, sizeof(n), cudaMemcpyHostToDevice, h->stream));
        CK(h, cudaStreamSynchronize(h->stream));
    }
    launch(k);   // warm-up
    CK(h, cudaEventRecord(e0, h->stream));
    for (int i = 0; i < reps; ++i) launch(k);
    CK(h, cudaEventRecord(e1, h->stream));
    CK(h, cudaEventSynchronize(e1));
    CKL(h);
    float t = 0;
    CK(h, cudaEventElapsedTime(&t, e0, e1));
    *ms = (double)t / reps;
    return RDXG_OK;
}

// ---------------------------------------------------------------------------------------
// Launch-shape planner: the counterpart of the reference's FFTW_MEASURE planning
// (fouriertransform.cpp:73-90), which times candidate transform plans once per size and
// keeps the fastest.  The candidates of the kernels that dominate a round -- k_eval (fused
// path: 512 or 384 threads), k_forward (general path) and k_adjoint (256 or 512 threads, 512
// or 1024 at N = 128) -- are their block sizes, which change no result (every element is
// computed by the same arithmetic whatever the block size), and, for the sizes with two
// two-stage radix plans (32, 64, 128; see PlanAlt), the plan, which changes the rounding of
// the transforms as FFTW's plans do.  The first solve of a handle measures the candidates on
// its loaded batch (the adjoint on a tenth of the patches, the share of a solve round that asks
// for gradients), unless a handle of the same geometry and batch size on the same device has
// already done so in this process (the tables below, the planner's wisdom); the plan is
// measured once per device, size and path, so every handle of a size uses the same.  FP64
// handles, the plain baseline form, have one shape.
// ---------------------------------------------------------------------------------------
struct ShapeKey {
    int device, N, fused, M, I, P;
    bool operator<(const ShapeKey& o) const {
        const int a[6] = {device, N, fused, M, I, P}, b[6] = {o.device, o.N, o.fused, o.M, o.I, o.P};
        return std::lexicographical_compare(a, a + 6, b, b + 6);
    }
};
struct ShapeChoice { int eval, fwd, adj; };
std::mutex& wisdom_mutex() {
    static std::mutex m;
    return m;
}
std::map<ShapeKey, ShapeChoice>& wisdom() {
    static std::map<ShapeKey, ShapeChoice> w;
    return w;
}
ShapeKey shape_key(const rdxg_solver* h) { return ShapeKey{h->geo.device, h->N, h->fused ? 1 : 0, h->M, h->I, h->P}; }

// The radix plans of the FFTs: R1 of plan 0 (Plan<N>) and plan 1 (PlanAlt<N>, 0 where N has none).
int radix_of(int N, int plan) {
    switch (N) {
        case 32: return plan ? PlanAlt<32>::R1 : Plan<32>::R1;
        case 64: return plan ? PlanAlt<64>::R1 : Plan<64>::R1;
        case 88: return plan ? 0 : Plan<88>::R1;
        case 128: return plan ? PlanAlt<128>::R1 : Plan<128>::R1;
        default: return 0;
    }
}

// The radix plan is chosen once per device, size and path in a process (the first handle
// measures it, every later one takes it), so that handles of one size -- a patch alone, in a
// batch, in a ragged batch -- give the same bits; the block sizes, which change no result, are
// chosen per geometry and batch size.
struct PlanKey {
    int device, N, fused;
    bool operator<(const PlanKey& o) const {
        const int a[3] = {device, N, fused}, b[3] = {o.device, o.N, o.fused};
        return std::lexicographical_compare(a, a + 3, b, b + 3);
    }
};
std::map<PlanKey, ShapeChoice>& plan_wisdom() {
    static std::map<PlanKey, ShapeChoice> w;
    return w;
}
PlanKey plan_key(const rdxg_solver* h) { return PlanKey{h->geo.device, h->N, h->fused ? 1 : 0}; }

// Measures the variants of every tuned kernel of the handle's path -- block size (bit 0 of
// the variant) and radix plan (bit 1), the plan only where none is fixed for this size yet --
// and keeps the fastest.  ms (or null): [6] eval (default, alternative block size),
// forward (...), adjoint (...) with the plan kept; 0 where a kernel is not tuned on this path.
int threads_of(const rdxg_solver* h, int family, int variant);

int plan_shapes(rdxg_solver* h, int reps, double* ms) {
    double t[6] = {0, 0, 0, 0, 0, 0};
    if (h->fp64) {
        h->shapeEval = h->shapeFwd = h->shapeAdj = 0;
        if (ms) std::memcpy(ms, t, sizeof(t));
        return RDXG_OK;
    }
    int fixedPlan[3] = {-1, -1, -1};
    {
        std::lock_guard<std::mutex> lock(wisdom_mutex());
        auto it = plan_wisdom().find(plan_key(h));
        if (it != plan_wisdom().end()) {
            fixedPlan[0] = it->second.eval >> 1; fixedPlan[1] = it->second.fwd >> 1; fixedPlan[2] = it->second.adj >> 1;
        }
    }
    CK(h, cudaMemsetAsync(h->dAlphaEff, 0, (size_t)h->P * h->I * h->M * sizeof(float), h->stream));
    cudaEvent_t e0, e1;
    CK(h, cudaEventCreate(&e0));
    CK(h, cudaEventCreate(&e1));
    int* field[3] = {&h->shapeEval, &h->shapeFwd, &h->shapeAdj};
    const bool used[3] = {h->fused, !h->fused, true};
    const int which[3] = {0, 0, 3};
    // a solve round evaluates every active patch but takes the gradients of about one in ten
    // (the others are in their line searches): the adjoint is timed on such a list, of at least
    // 24 patches (on shorter lists the block sizes time alike within the noise, while the
    // larger one is faster in a solve whose handles run side by side)
    const int nGrad[3] = {0, 0, std::min(h->P, std::max(24, (h->P + 9) / 10))};
    const bool altPlan = radix_of(h->N, 1) != 0;
    int r = RDXG_OK;
    double all[3][4] = {};
    for (int f = 0; f < 3 && !r; ++f) {
        if (!used[f]) { *field[f] = 0; continue; }
        double* tv = all[f];
        bool avail[4];
        for (int v = 0; v < 4; ++v) {
            const int plan = v >> 1;
            avail[v] = threads_of(h, f, v & 1) != 0 && (plan == 0 || altPlan) &&
                       (fixedPlan[f] < 0 || plan == fixedPlan[f]);
        }
        // each candidate timed three times, alternating, the fastest of each kept (a single
        // measurement of these sub-millisecond launches is at the mercy of the clock ramp)
        for (int rep = 0; rep < 3 && !r; ++rep) {
            for (int v = 0; v < 4 && !r; ++v) {
                if (!avail[v]) continue;
                *field[f] = v;
                double ms1 = 0;
                r = time_kernel(h, which[f], reps, e0, e1, &ms1, nGrad[f]);
                if (rep == 0 || ms1 < tv[v]) tv[v] = ms1;
            }
        }
        int best = -1;
        for (int v = 0; v < 4; ++v)
            if (avail[v] && (best < 0 || tv[v] < tv[best])) best = v;
        *field[f] = best < 0 ? 0 : best;
        const int plan = *field[f] >> 1;
        t[2 * f] = tv[2 * plan];
        t[2 * f + 1] = avail[2 * plan + 1] ? tv[2 * plan + 1] : 0.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r) return r;
    h->dirty = true;     // the timed kernels overwrote per-image state: the solve re-initialises
    {
        std::lock_guard<std::mutex> lock(wisdom_mutex());
        wisdom()[shape_key(h)] = ShapeChoice{h->shapeEval, h->shapeFwd, h->shapeAdj};
        plan_wisdom().emplace(plan_key(h), ShapeChoice{h->shapeEval, h->shapeFwd, h->shapeAdj});
    }
    if (getenv("RDXG_VERBOSE"))
        fprintf(stderr, "launch shapes (N %d, P %d): eval %d [%.3f %.3f | %.3f %.3f ms], forward %d [%.3f %.3f | %.3f "
                "%.3f], adjoint %d [%.3f %.3f | %.3f %.3f] (plan 0: threads, alternative threads | plan 1)\n", h->N,
                h->P, h->shapeEval, all[0][0], all[0][1], all[0][2], all[0][3], h->shapeFwd, all[1][0], all[1][1],
                all[1][2], all[1][3], h->shapeAdj, all[2][0], all[2][1], all[2][2], all[2][3]);
    if (ms) std::memcpy(ms, t, sizeof(t));
    return RDXG_OK;
}

// The first solve of a handle: shapes from the planner's table, or measured.
int plan_shapes_once(rdxg_solver* h) {
    if (h->tune != 1 || h->tuned) return RDXG_OK;
    h->tuned = true;
    {
        std::lock_guard<std::mutex> lock(wisdom_mutex());
        auto it = wisdom().find(shape_key(h));
        if (it != wisdom().end()) {
            h->shapeEval = it->second.eval; h->shapeFwd = it->second.fwd; h->shapeAdj = it->second.adj;
            return RDXG_OK;
        }
    }
    return plan_shapes(h, 3, nullptr);
}

// threads per block of a variant (bit 0: the alternative block size), 0 where the kernel is
// not used on the handle's path
int threads_of(const rdxg_solver* h, int family, int variant) {
    const int alt = variant & 1;
    if (family == 0) return h->fused ? (alt ? kEvalThreadsAlt : kEvalThreads) : 0;
    if (family == 1 && h->fused) return 0;
    const int base = h->N >= 128 ? 512 : 256;
    return (alt && !h->fp64) ? 2 * base : base;
}

}  // namespace
}  // extern "C++"

int rdxg_profile_kernels(rdxg_solver* h, int32_t reps, double* ms) {
    if (!h || !ms || reps < 1) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    cudaEvent_t e0, e1;
    CK(h, cudaEventCreate(&e0));
    CK(h, cudaEventCreate(&e1));
    int r = RDXG_OK;
    for (int k = 0; k < 5 && !r; ++k) r = time_kernel(h, k, reps, e0, e1, &ms[k]);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return r;
}

int rdxg_autotune(rdxg_solver* h, int32_t reps, rdxg_launch_shape* chosen, double* ms) {
    if (!h || reps < 1) return RDXG_ERR_ARG;
    if (!h->loaded) { h->err = "no patches loaded"; return RDXG_ERR_STATE; }
    int r = plan_shapes(h, reps, ms);
    if (r) return r;
    h->tuned = true;
    h->tune = 1;
    return rdxg_get_launch_shape(h, chosen);
}

int rdxg_set_launch_shape(rdxg_solver* h, const rdxg_launch_shape* shape) {
    if (!h || !shape) return RDXG_ERR_ARG;
    int v[3] = {h->shapeEval, h->shapeFwd, h->shapeAdj};
    const int32_t want[3] = {shape->eval_threads, shape->forward_threads, shape->adjoint_threads};
    const int32_t wantRadix[3] = {shape->eval_radix, shape->forward_radix, shape->adjoint_radix};
    for (int f = 0; f < 3; ++f) {
        if (want[f] == 0 && wantRadix[f] == 0) continue;
        if (threads_of(h, f, 0) == 0) {
            h->err = std::string(f == 0 ? "k_eval" : "k_forward") + " is not used on this handle's path";
            return RDXG_ERR_ARG;
        }
        int tv = v[f] & 1, pv = v[f] >> 1;
        if (want[f] != 0) {
            if (want[f] == threads_of(h, f, 0)) tv = 0;
            else if (want[f] == threads_of(h, f, 1)) tv = 1;
            else {
                h->err = "launch shape " + std::to_string(want[f]) + " is not compiled for this kernel (" +
                         std::to_string(threads_of(h, f, 0)) + " or " + std::to_string(threads_of(h, f, 1)) + ")";
                return RDXG_ERR_ARG;
            }
        }
        if (wantRadix[f] != 0) {
            if (wantRadix[f] == radix_of(h->N, 0)) pv = 0;
            else if (!h->fp64 && wantRadix[f] == radix_of(h->N, 1)) pv = 1;
            else {
                h->err = "radix " + std::to_string(wantRadix[f]) + " is not a plan of size " + std::to_string(h->N);
                return RDXG_ERR_ARG;
            }
        }
        v[f] = tv | (pv << 1);
    }
    if (shape->solver_form < 0 || shape->solver_form > 2) {
        h->err = "solver_form is 1 (staged) or 2 (global memory)";
        return RDXG_ERR_ARG;
    }
    if (shape->solver_form) h->cgForm = shape->solver_form;
    bool pinned = false;
    for (int f = 0; f < 3; ++f) pinned = pinned || want[f] != 0 || wantRadix[f] != 0;
    h->shapeEval = v[0]; h->shapeFwd = v[1]; h->shapeAdj = v[2];
    if (pinned) h->tune = 0;
    return RDXG_OK;
}

int rdxg_get_launch_shape(const rdxg_solver* h, rdxg_launch_shape* shape) {
    if (!h || !shape) return RDXG_ERR_ARG;
    shape->eval_threads = threads_of(h, 0, h->shapeEval);
    shape->forward_threads = threads_of(h, 1, h->shapeFwd);
    shape->adjoint_threads = threads_of(h, 2, h->shapeAdj);
    shape->eval_radix = shape->eval_threads ? radix_of(h->N, h->shapeEval >> 1) : 0;
    shape->forward_radix = shape->forward_threads ? radix_of(h->N, h->shapeFwd >> 1) : 0;
    shape->adjoint_radix = radix_of(h->N, h->shapeAdj >> 1);
    int32_t stage = 0, map = 0;
    size_t bytes = 0;
    cg_stage_choice(h, &stage, &map, &bytes);
    shape->solver_form = stage ? 1 : 2;
    return RDXG_OK;
}

int rdxg_debug_set(rdxg_solver* h, int32_t which, const void* in, size_t bytes) {
    if (!h || !in) return RDXG_ERR_ARG;
    switch (which) {
        case 0: {
            // the tensor-core expansion's status word, as a wait that gave up leaves it
            if (!h->dTcStatus || bytes != sizeof(int32_t)) return RDXG_ERR_ARG;
            CK(h, cudaMemcpyAsync(h->dTcStatus, in, sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
            CK(h, cudaStreamSynchronize(h->stream));
            return RDXG_OK;
        }
        default: return RDXG_ERR_ARG;
    }
}

int rdxg_debug_copy(rdxg_solver* h, int32_t which, void* out, size_t bytes) {
    if (!h || !out) return RDXG_ERR_ARG;
    const size_t G = (size_t)h->P * h->I, N2 = (size_t)h->N * h->N, PO = (size_t)h->P * h->nObj;
    const size_t cxs = h->fp64 ? 16 : 8;
    CK(h, cudaStreamSynchronize(h->stream));
    switch (which) {
        case 0: if (bytes < G * N2 * cxs) return RDXG_ERR_ARG; CK(h, cudaMemcpy(out, h->dD, G * N2 * cxs, cudaMemcpyDeviceToHost)); break;
        case 1:
            if (bytes < G * N2 * cxs) return RDXG_ERR_ARG;
            if (!h->dS) { h->err = "the OTFs are not kept (recomputed transforms)"; return RDXG_ERR_STATE; }
            CK(h, cudaMemcpy(out, h->dS, G * N2 * cxs, cudaMemcpyDeviceToHost));
            break;
        case 2: if (bytes < PO * 8) return RDXG_ERR_ARG; CK(h, cudaMemcpy(out, h->dGamma, PO * 8, cudaMemcpyDeviceToHost)); break;
        case 3: {
            if (bytes < G * 3 * 8) return RDXG_ERR_ARG;
            std::vector<double> a(G), b(G), c(G);
            CK(h, cudaMemcpy(a.data(), h->dMean, G * 8, cudaMemcpyDeviceToHost));
            CK(h, cudaMemcpy(b.data(), h->dStd, G * 8, cudaMemcpyDeviceToHost));
            CK(h, cudaMemcpy(c.data(), h->dNoise, G * 8, cudaMemcpyDeviceToHost));
            double* o = (double*)out;
            for (size_t g = 0; g < G; ++g) { o[3 * g] = a[g]; o[3 * g + 1] = b[g]; o[3 * g + 2] = c[g]; }
            break;
        }
        case 4: if (bytes < PO * N2 * cxs) return RDXG_ERR_ARG; CK(h, cudaMemcpy(out, h->dO, PO * N2 * cxs, cudaMemcpyDeviceToHost)); break;
        case 5: if (bytes < G * 2 * 4) return RDXG_ERR_ARG; CK(h, cudaMemcpy(out, h->dShift, G * 8, cudaMemcpyDeviceToHost)); break;
        case 6: {
            const size_t nb = G * (size_t)h->n * h->n * sizeof(float);
            if (!h->dPhiImg || (!h->fused && !h->tcPlan.valid) || bytes < nb) return RDXG_ERR_ARG;
            CK(h, cudaMemcpy(out, h->dPhiImg, nb, cudaMemcpyDeviceToHost));
            break;
        }
        case 7: {
            if (bytes < sizeof(int64_t)) return RDXG_ERR_ARG;
            const int64_t n = (int64_t)h->allocs.size();
            std::memcpy(out, &n, sizeof(n));
            break;
        }
        case 8: {
            if (bytes < sizeof(int64_t)) return RDXG_ERR_ARG;
            const int64_t n = (int64_t)h->allocBytes;
            std::memcpy(out, &n, sizeof(n));
            break;
        }
        default: return RDXG_ERR_ARG;
    }
    return RDXG_OK;
}

}  // extern "C"
