// rdxg_solver.hpp -- C++ shim with the shape of redux's momfbd::Solver over the C ABI.
//
// Mirrors include/redux/momfbd/solver.hpp:86-179 (ISP-SST/redux): construction once per job
// (Solver::Solver + Solver::init), run(PatchData) per patch (Solver::run, solver.cpp:330-580),
// metric() at the current alpha (Solver::metric, solver.cpp:763-817), applyAlpha(a)
// (solver.cpp:219-225) and the public alpha vector.  The job-side types of the reference
// (MomfbdJob, PatchData, ObjectData) are represented by the plain structs below, which hold
// what Solver::run reads and writes: the float32 channel cutouts in, the mode coefficients,
// metric history, final metric and restored objects out (solver.cpp:551-566), with the PSFs,
// convolved objects and residuals that Object::restorePatch saves when asked (object.cpp:335-383).
//
// Errors: every failing rdxg_* call throws std::runtime_error with rdxg_last_error()
// (the reference throws std::logic_error for a corrupt constraint set, solver.cpp:102-110,
// and only logs run-time failures).  Header only; link with libredux_gb300.so.
#ifndef RDXG_SOLVER_HPP
#define RDXG_SOLVER_HPP

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "rdxg.h"

namespace rdxg {

// The GlobalCfg fields Solver::run reads (config.hpp:196-228), with the reference defaults
// of config.cpp:629-636.
struct Settings {
    int32_t modeStart = 5;          // MODE_START
    int32_t modeStep = 5;           // MODE_STEP
    int32_t maxIterations = 500;    // MAX_ITER
    int32_t minIterations = 5;      // MIN_ITER
    int32_t targetIterations = 3;   // N_DONE_ITER
    bool finiteDifferenceFirst = true;
    double ftol = 1e-3;             // FTOL
    double eps = 1e-10;             // EPS
    int32_t maxMetrics = 1024;      // capacity of the metric history per patch
    bool restore = true;            // restore the objects after the solve
    bool noFilter = false;          // RF_NO_FILTER
    bool fitPlane = false;          // RF_FIT_PLANE
    std::vector<double> regAlphaWeights;   // [I][M] Solver::regAlphaWeights, empty for REG_ALPHA = 0
    // further outputs of the restoration (Object::saveMask): RDXG_RESTORE_PSF,
    // RDXG_RESTORE_PSF_AVG, RDXG_RESTORE_COBJ, RDXG_RESTORE_RESIDUAL
    int32_t saveMask = 0;
};

// What Solver::run takes from and gives back to PatchData (data.hpp:144-196).
struct PatchData {
    std::vector<float> cutouts;          // [I][cutout][cutout] channel images with margins
    std::vector<double> residualAlpha;   // [I][2] (y, x) residual tilt, or empty
    std::vector<double> fixedGamma;      // [nObj] fixed regularisation, or empty
    std::vector<double> initAlpha;       // [I][M] initial coefficients (INIT_FILES), or empty
    // results
    std::vector<double> alpha;           // [I][M] mode coefficients (waveFronts.alpha)
    std::vector<double> metrics;         // metric history (PatchData::metrics)
    double finalMetric = 0;              // PatchData::finalMetric
    int32_t iterations = 0;
    int32_t status = 0;                  // 0 ok, 1 gave up after too many failures
    std::vector<float> objects;          // [nObj][ps][ps] restored objects (ObjectData::img)
    std::vector<float> psf;              // [I][ps][ps] or, with RDXG_RESTORE_PSF_AVG, [nObj][ps][ps]
    std::vector<float> cobj;             // [I][ps][ps] convolved objects (ObjectData::cobj)
    std::vector<float> res;              // [I][ps][ps] residuals (ObjectData::res)
};

class Solver {
public:
    // Solver(MomfbdJob&, io_service&, nThreads) + init(): the static job data and the
    // geometry; frequencyCutoff: [nObj] Object::frequencyCutoff (for the restoration).
    Solver(const rdxg_geometry& geometry, const rdxg_static& statics, const Settings& settings,
           std::vector<double> frequencyCutoff)
        : geo_(geometry), set_(settings), fc_(std::move(frequencyCutoff)) {
        check(rdxg_create(&geo_, &statics, &h_), "rdxg_create");
        if (set_.fitPlane) check(rdxg_set_fit_plane(h_, 1), "rdxg_set_fit_plane");
        if (!set_.regAlphaWeights.empty()) {
            if (set_.regAlphaWeights.size() != (size_t)geo_.n_images * geo_.n_modes)
                throw std::runtime_error("rdxg::Solver: regAlphaWeights size mismatch");
            check(rdxg_set_reg_alpha(h_, set_.regAlphaWeights.data()), "rdxg_set_reg_alpha");
        }
        if ((int)fc_.size() != geo_.n_objects) fc_.assign(geo_.n_objects, geo_.otf_size / 2.0);
        alpha.assign((size_t)geo_.n_images * geo_.n_modes, 0.0);
    }
    ~Solver() { rdxg_destroy(h_); }
    Solver(const Solver&) = delete;
    Solver& operator=(const Solver&) = delete;

    void init() {}   // done by the constructor (the reference's init sleeps >= 1 s)

    // Solver::run for one patch (a batch of one).
    void run(PatchData& data) {
        std::vector<PatchData*> one{&data};
        run(one);
    }

    // The same for several patches at once (one batch, one device pass per round).
    void run(const std::vector<PatchData*>& batch) {
        const int P = (int)batch.size();
        if (P < 1 || P > geo_.max_patches) throw std::runtime_error("rdxg::Solver::run: batch size out of range");
        const size_t I = geo_.n_images, cs = geo_.cutout_size, M = geo_.n_modes;
        std::vector<float> cut(P * I * cs * cs);
        std::vector<double> res, gam;
        const bool haveRes = !batch[0]->residualAlpha.empty(), haveGam = !batch[0]->fixedGamma.empty();
        if (haveRes) res.resize(P * I * 2);
        if (haveGam) gam.resize((size_t)P * geo_.n_objects);
        for (int p = 0; p < P; ++p) {
            const PatchData& d = *batch[p];
            if (d.cutouts.size() != I * cs * cs) throw std::runtime_error("rdxg::Solver::run: cutout size mismatch");
            std::copy(d.cutouts.begin(), d.cutouts.end(), cut.begin() + p * I * cs * cs);
            if (haveRes) std::copy(d.residualAlpha.begin(), d.residualAlpha.end(), res.begin() + p * I * 2);
            if (haveGam) std::copy(d.fixedGamma.begin(), d.fixedGamma.end(), gam.begin() + (size_t)p * geo_.n_objects);
        }
        check(rdxg_set_patches(h_, P, cut.data(), haveRes ? res.data() : nullptr, haveGam ? gam.data() : nullptr),
              "rdxg_set_patches");
        if (!batch[0]->initAlpha.empty()) {      // Solver::loadInit: a warm start for the batch
            std::vector<double> init(P * I * M);
            for (int p = 0; p < P; ++p) {
                if (batch[p]->initAlpha.size() != I * M) throw std::runtime_error("rdxg::Solver::run: initAlpha size mismatch");
                std::copy(batch[p]->initAlpha.begin(), batch[p]->initAlpha.end(), init.begin() + p * I * M);
            }
            check(rdxg_set_initial_alpha(h_, init.data()), "rdxg_set_initial_alpha");
        }
        rdxg_solve_params prm{};
        prm.mode_start = set_.modeStart;
        prm.mode_step = set_.modeStep;
        prm.max_iterations = set_.maxIterations;
        prm.min_iterations = set_.minIterations;
        prm.target_iterations = set_.targetIterations;
        prm.fd_first = set_.finiteDifferenceFirst ? 1 : 0;
        prm.max_metrics = set_.maxMetrics;
        prm.check_every = 8;
        prm.ftol = set_.ftol;
        prm.eps = set_.eps;
        std::vector<double> al(P * I * M);
        std::vector<rdxg_patch_report> rep(P);
        std::vector<double> met((size_t)P * set_.maxMetrics);
        check(rdxg_solve(h_, &prm, al.data(), rep.data(), met.data()), "rdxg_solve");
        std::vector<float> obj, psf, cobj, resid;
        const size_t ps = geo_.patch_size, nObj = geo_.n_objects, ps2 = ps * ps;
        const int32_t mask = set_.restore ? set_.saveMask : 0;
        const size_t nPsf = (mask & RDXG_RESTORE_PSF_AVG) ? nObj : (mask & RDXG_RESTORE_PSF) ? I : 0;
        if (set_.restore) {
            obj.resize(P * nObj * ps2);
            psf.resize(P * nPsf * ps2);
            if (mask & RDXG_RESTORE_COBJ) cobj.resize(P * I * ps2);
            if (mask & RDXG_RESTORE_RESIDUAL) resid.resize(P * I * ps2);
            check(rdxg_restore_ex(h_, al.data(), fc_.data(), set_.noFilter ? 1 : 0, mask, obj.data(),
                                  psf.empty() ? nullptr : psf.data(), cobj.empty() ? nullptr : cobj.data(),
                                  resid.empty() ? nullptr : resid.data()),
                  "rdxg_restore_ex");
        }
        for (int p = 0; p < P; ++p) {
            PatchData& d = *batch[p];
            d.alpha.assign(al.begin() + p * I * M, al.begin() + (p + 1) * I * M);
            const int nm = rep[p].n_metrics < set_.maxMetrics ? rep[p].n_metrics : set_.maxMetrics;
            d.metrics.assign(met.begin() + (size_t)p * set_.maxMetrics, met.begin() + (size_t)p * set_.maxMetrics + nm);
            d.finalMetric = rep[p].final_metric;
            d.iterations = rep[p].iterations;
            d.status = rep[p].status;
            if (set_.restore) d.objects.assign(obj.begin() + p * nObj * ps2, obj.begin() + (p + 1) * nObj * ps2);
            auto part = [&](const std::vector<float>& v, size_t per, std::vector<float>& dst) {
                if (v.empty()) dst.clear();
                else dst.assign(v.begin() + p * per, v.begin() + (p + 1) * per);
            };
            part(psf, nPsf * ps2, d.psf);
            part(cobj, I * ps2, d.cobj);
            part(resid, I * ps2, d.res);
        }
        alpha.assign(al.begin() + (P - 1) * I * M, al.end());
        loaded_ = P;
    }

    // Solver::applyAlpha(a): the coefficients at which metric() evaluates ([I][M]).
    template <typename T> void applyAlpha(const T* a) {
        for (size_t i = 0; i < alpha.size(); ++i) alpha[i] = (double)a[i];
    }
    void applyAlpha() {}

    // Solver::metric() at the current alpha for the last patch loaded by run().
    double metric() {
        if (loaded_ < 1) throw std::runtime_error("rdxg::Solver::metric: no patch loaded");
        std::vector<double> a((size_t)loaded_ * alpha.size()), m(loaded_);
        for (int p = 0; p < loaded_; ++p) std::copy(alpha.begin(), alpha.end(), a.begin() + p * alpha.size());
        check(rdxg_metric(h_, a.data(), m.data()), "rdxg_metric");
        return m[loaded_ - 1];
    }

    rdxg_solver* handle() { return h_; }

    std::vector<double> alpha;   // [I][M], public as in the reference

private:
    void check(int r, const char* what) {
        if (r != RDXG_OK) {
            const char* e = h_ ? rdxg_last_error(h_) : "";
            throw std::runtime_error(std::string(what) + " failed (status " + std::to_string(r) + "): " + (e ? e : ""));
        }
    }
    rdxg_geometry geo_;
    Settings set_;
    std::vector<double> fc_;
    rdxg_solver* h_ = nullptr;
    int loaded_ = 0;
};

}  // namespace rdxg

#endif  // RDXG_SOLVER_HPP
