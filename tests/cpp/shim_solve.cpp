// Test driver for include/rdxg_solver.hpp: reads a job and patches written by
// tests/test_cpp_shim.py (raw little-endian arrays, one file each), solves them through
// rdxg::Solver and writes alpha, metrics, reports, restored objects, PSFs, convolved objects
// and residuals back.
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "rdxg_solver.hpp"

template <typename T>
static std::vector<T> load(const std::string& dir, const char* name, bool required = true) {
    std::vector<T> v;
    FILE* f = std::fopen((dir + "/" + name).c_str(), "rb");
    if (!f) {
        if (required) throw std::runtime_error(std::string("missing ") + name);
        return v;
    }
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    v.resize((size_t)n / sizeof(T));
    if (n && std::fread(v.data(), sizeof(T), v.size(), f) != v.size()) throw std::runtime_error("short read");
    std::fclose(f);
    return v;
}

template <typename T>
static void save(const std::string& dir, const char* name, const std::vector<T>& v) {
    FILE* f = std::fopen((dir + "/" + name).c_str(), "wb");
    if (!f) throw std::runtime_error(std::string("cannot write ") + name);
    std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

int main(int argc, char** argv) {
    if (argc != 2) {
        std::fprintf(stderr, "usage: shim_solve <dir>\n");
        return 2;
    }
    const std::string dir = argv[1];
    try {
        const auto gi = load<int32_t>(dir, "geom.i32");
        rdxg_geometry g{gi[0], gi[1], gi[2], gi[3], gi[4], gi[5], gi[6], gi[7], gi[8], gi[9], gi[10], gi[11], gi[12], gi[13]};
        const auto modes = load<double>(dir, "modes.f64"), pupil = load<double>(dir, "pupil.f64");
        const auto psup = load<int32_t>(dir, "pupil_support.i32"), osup = load<int32_t>(dir, "otf_support.i32");
        const auto iobj = load<int32_t>(dir, "image_object.i32"), ich = load<int32_t>(dir, "image_channel.i32");
        const auto phif = load<double>(dir, "phi_fixed.f64"), ow = load<double>(dir, "object_weight.f64");
        const auto og = load<double>(dir, "object_grad_step.f64"), win = load<double>(dir, "window.f64");
        const auto nwin = load<double>(dir, "noise_window.f64");
        const auto nsr = load<int32_t>(dir, "ns_rows.i32"), nsc = load<int32_t>(dir, "ns_cols.i32");
        const auto nsv = load<double>(dir, "ns_vals.f64"), jac = load<double>(dir, "tilt_jacobian.f64");
        rdxg_static s{};
        s.modes = modes.data(); s.pupil = pupil.data();
        s.n_pupil_support = (int32_t)psup.size(); s.pupil_support = psup.data();
        s.n_otf_support = (int32_t)osup.size(); s.otf_support = osup.data();
        s.image_object = iobj.data(); s.image_channel = ich.data(); s.phi_fixed = phif.data();
        s.object_weight = ow.data(); s.object_grad_step = og.data();
        s.window = win.data(); s.noise_window = nwin.data();
        s.ns_nnz = (int64_t)nsv.size(); s.ns_rows = nsr.data(); s.ns_cols = nsc.data(); s.ns_vals = nsv.data();
        s.tilt_jacobian = jac.data();
        const auto sv = load<double>(dir, "settings.f64");
        rdxg::Settings set;
        set.modeStart = (int32_t)sv[0]; set.modeStep = (int32_t)sv[1]; set.maxIterations = (int32_t)sv[2];
        set.minIterations = (int32_t)sv[3]; set.targetIterations = (int32_t)sv[4];
        set.finiteDifferenceFirst = sv[5] != 0; set.ftol = sv[6]; set.eps = sv[7]; set.maxMetrics = (int32_t)sv[8];
        set.restore = true;
        if (sv.size() > 9) set.saveMask = (int32_t)sv[9];
        // optional: FIT_PLANE, REG_ALPHA weights, warm-start coefficients
        const auto flags = load<int32_t>(dir, "fit_plane.i32", false);
        set.fitPlane = !flags.empty() && flags[0] != 0;
        set.regAlphaWeights = load<double>(dir, "reg_alpha.f64", false);
        const auto init = load<double>(dir, "init_alpha.f64", false);
        rdxg::Solver solver(g, s, set, load<double>(dir, "fc.f64"));
        solver.init();
        const auto cut = load<float>(dir, "cutouts.f32");
        const auto gam = load<double>(dir, "fixed_gamma.f64", false);
        const size_t per = (size_t)g.n_images * g.cutout_size * g.cutout_size;
        const int P = (int)(cut.size() / per);
        std::vector<rdxg::PatchData> pd(P);
        std::vector<rdxg::PatchData*> batch;
        for (int p = 0; p < P; ++p) {
            pd[p].cutouts.assign(cut.begin() + p * per, cut.begin() + (p + 1) * per);
            if (!gam.empty()) pd[p].fixedGamma.assign(gam.begin() + (size_t)p * g.n_objects, gam.begin() + (size_t)(p + 1) * g.n_objects);
            const size_t nPar = (size_t)g.n_images * g.n_modes;
            if (!init.empty()) pd[p].initAlpha.assign(init.begin() + p * nPar, init.begin() + (p + 1) * nPar);
            batch.push_back(&pd[p]);
        }
        solver.run(batch);
        std::vector<double> alpha, metrics, rep;
        std::vector<float> obj, psf, cobj, res;
        for (int p = 0; p < P; ++p) {
            psf.insert(psf.end(), pd[p].psf.begin(), pd[p].psf.end());
            cobj.insert(cobj.end(), pd[p].cobj.begin(), pd[p].cobj.end());
            res.insert(res.end(), pd[p].res.begin(), pd[p].res.end());
            alpha.insert(alpha.end(), pd[p].alpha.begin(), pd[p].alpha.end());
            std::vector<double> m(set.maxMetrics, 0.0);
            std::copy(pd[p].metrics.begin(), pd[p].metrics.end(), m.begin());
            metrics.insert(metrics.end(), m.begin(), m.end());
            rep.push_back(pd[p].finalMetric);
            rep.push_back(pd[p].iterations);
            rep.push_back((double)pd[p].metrics.size());
            obj.insert(obj.end(), pd[p].objects.begin(), pd[p].objects.end());
        }
        // Solver::metric at the final alpha of the last patch
        solver.applyAlpha(pd[P - 1].alpha.data());
        rep.push_back(solver.metric());
        save(dir, "alpha.out.f64", alpha);
        save(dir, "metrics.out.f64", metrics);
        save(dir, "report.out.f64", rep);
        save(dir, "objects.out.f32", obj);
        save(dir, "psf.out.f32", psf);
        save(dir, "cobj.out.f32", cobj);
        save(dir, "res.out.f32", res);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "shim_solve: %s\n", e.what());
        return 1;
    }
    return 0;
}
