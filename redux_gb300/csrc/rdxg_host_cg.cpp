// Host driver of the per-patch optimiser state machine (rdxg_cg_minimize).
//
// The same machine as the device kernel, driven sequentially with caller-supplied
// metric and gradient callbacks; the vector operations follow the reference's GSL calls
// (gsl_blas_dnrm2 with its scaled sum of squares, gsl_blas_ddot, daxpy), so the sequence
// of evaluations can be compared exactly with a sequential restatement of
// conjugate_rdx_iterate (src/lib/util/gsl/conjugate_gradient.cpp:128-256).
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/rdxg.h"
#include "cg_machine.h"

using namespace rdxg;

namespace {

struct HostVec {
    int n;
    void copy(double* d, const double* s) { std::memcpy(d, s, sizeof(double) * (size_t)n); }
    void zero(double* d) { std::memset(d, 0, sizeof(double) * (size_t)n); }
    double nrm2(const double* v) {
        double scale = 0.0, ssq = 1.0;
        if (n == 1) return std::fabs(v[0]);
        for (int i = 0; i < n; ++i) {
            if (v[i] != 0.0) {
                const double ax = std::fabs(v[i]);
                if (scale < ax) {
                    ssq = 1.0 + ssq * (scale / ax) * (scale / ax);
                    scale = ax;
                } else {
                    ssq += (ax / scale) * (ax / scale);
                }
            }
        }
        return scale * std::sqrt(ssq);
    }
    double dot(const double* a, const double* b) {
        double s = 0;
        for (int i = 0; i < n; ++i) s += a[i] * b[i];
        return s;
    }
    double pr_update(double* g0, const double* g) {
        double s = 0;
        for (int i = 0; i < n; ++i) {
            const double t = g0[i] - g[i];
            s += t * g[i];
            g0[i] = t;
        }
        return s;
    }
    void dir_update(double* p, const double* g, double beta) {
        for (int i = 0; i < n; ++i) p[i] = g[i] - beta * p[i];
    }
    void step(double* x1, const double* x, const double* p, double s) {
        for (int i = 0; i < n; ++i) {
            const double dx = 0.0 + s * p[i];
            x1[i] = x[i] + 1.0 * dx;
        }
    }
};

}  // namespace

extern "C" int rdxg_cg_minimize(int32_t n_free, int32_t n_modes, const rdxg_solve_params* s,
                                double grad_scale, rdxg_f_fn f, rdxg_df_fn df, rdxg_shift_fn shift,
                                void* user, double* x_out, rdxg_patch_report* report, double* metrics) {
    if (n_free < 1 || n_modes < 1 || !s || !f || !df) return RDXG_ERR_ARG;
    CgParams prm{};
    prm.n_free = n_free;
    prm.n_modes = n_modes;
    prm.mode_start = s->mode_start > 0 ? s->mode_start : 1;
    prm.mode_step = s->mode_step > 0 ? s->mode_step : 1;
    prm.max_iterations = s->max_iterations;
    prm.min_iterations = s->min_iterations;
    prm.target_iterations = s->target_iterations;
    prm.fd_first = s->fd_first;
    prm.max_fails = 3;
    prm.max_metrics = s->max_metrics;
    prm.ftol = s->ftol;
    prm.eps = s->eps;
    prm.grad_scale = grad_scale;
    prm.brent_tol = 0.1;
    prm.init_step = 1E-21;
    std::vector<double> buf(5 * (size_t)n_free, 0.0);
    double *x = buf.data(), *p = x + n_free, *g = p + n_free, *g0 = g + n_free, *x1 = g0 + n_free;
    CgState st;
    std::memset(&st, 0, sizeof(st));
    HostVec V{n_free};
    Machine<HostVec> m(prm, st, V, x, p, g, g0, x1, metrics);
    double fv = 0;
    for (;;) {
        const int rq = m.advance(fv);
        if (rq == REQ_F) {
            fv = f(x1, user);
        } else if (rq == REQ_DF) {
            df(x1, st.grad_method, st.mode_count, g, user);
        } else if (rq == REQ_SHIFT) {
            if (shift) shift(x1, user);
        } else {
            break;
        }
    }
    if (x_out) std::memcpy(x_out, x, sizeof(double) * (size_t)n_free);
    if (report) {
        report->initial_metric = st.initial_metric;
        report->final_metric = st.this_metric;
        report->iterations = st.total_iterations;
        report->status = st.status == ST_FAILURE ? 1 : 0;
        report->n_f_evals = st.n_f;
        report->n_df_evals = st.n_df;
        report->fail_count = st.fail_count;
        report->n_metrics = st.n_metrics;
    }
    return RDXG_OK;
}
