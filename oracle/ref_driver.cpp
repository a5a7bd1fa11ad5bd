// Driver of the reference's own compiled minimiser (oracle/_ref/libref_cg.so).
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/ to pin the conjugate-gradient iteration and the
// line search; the product never links or calls it.
//
// libref_cg.so is built (oracle/Makefile, target ref) from three parts:
//   * the reference's own sources, compiled where they lie in the ISP-SST/redux tree:
//       src/lib/util/gsl/conjugate_gradient.cpp  (conjugate_rdx_set/iterate 72-256, the GSL
//                                                 minimiser type multimin_fdfminimizer_conjugate_rdx)
//       src/lib/math/helpers.cpp                 (bracket 58-129, brent 133-215)
//     with the reference's headers (include/redux/util/gsl.hpp for rdx_fdf,
//     include/redux/math/helpers.hpp, include/redux/constants.hpp);
//   * oracle/ref_shim/: the part of GSL's public API those files use (gsl_vector, three
//     level-1 BLAS calls, the multimin fdf framework), a stand-in for Boost's numeric_cast and
//     an empty stringutil.hpp -- GSL and Boost are not installed here;
//   * this file: the GSL calls restated (GSL >= 1.16, multimin/fdfminimizer.c and its
//     reference CBLAS nrm2/dot/axpy), and the stage loop of Solver::run (solver.cpp:405-537)
//     around gsl_multimin_fdfminimizer_iterate, driving caller callbacks instead of a patch.
// The loop is a restatement (Solver::run needs the whole library); the iteration, bracketing
// and Brent search it calls are the reference's compiled code.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>

#include <gsl/gsl_blas.h>
#include <gsl/gsl_multimin.h>

#include "redux/util/gsl.hpp"

// ---- GSL vector and BLAS (unit stride) ----
gsl_vector* gsl_vector_calloc(size_t n) {
    gsl_vector* v = static_cast<gsl_vector*>(std::malloc(sizeof(gsl_vector)));
    if (!v) return nullptr;
    v->size = n;
    v->stride = 1;
    v->data = static_cast<double*>(std::calloc(n ? n : 1, sizeof(double)));
    v->block = nullptr;
    v->owner = 1;
    if (!v->data) {
        std::free(v);
        return nullptr;
    }
    return v;
}
gsl_vector* gsl_vector_alloc(size_t n) { return gsl_vector_calloc(n); }
void gsl_vector_free(gsl_vector* v) {
    if (!v) return;
    std::free(v->data);
    std::free(v);
}
int gsl_vector_memcpy(gsl_vector* dest, const gsl_vector* src) {
    if (dest->size != src->size) GSL_ERROR("vector lengths are not equal", GSL_FAILURE);
    std::memcpy(dest->data, src->data, sizeof(double) * src->size);
    return GSL_SUCCESS;
}
void gsl_vector_set_zero(gsl_vector* v) {
    for (size_t i = 0; i < v->size; ++i) v->data[i] = 0.0;
}
// cblas_dnrm2: scaled sum of squares
double gsl_blas_dnrm2(const gsl_vector* x) {
    const size_t n = x->size;
    const double* X = x->data;
    if (n == 0) return 0.0;
    if (n == 1) return std::fabs(X[0]);
    double scale = 0.0, ssq = 1.0;
    for (size_t i = 0; i < n; ++i) {
        const double v = X[i];
        if (v != 0.0) {
            const double ax = std::fabs(v);
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
// cblas_ddot: a running sum in index order
int gsl_blas_ddot(const gsl_vector* x, const gsl_vector* y, double* result) {
    if (x->size != y->size) GSL_ERROR("invalid length", GSL_FAILURE);
    double r = 0.0;
    for (size_t i = 0; i < x->size; ++i) r += x->data[i] * y->data[i];
    *result = r;
    return GSL_SUCCESS;
}
// cblas_daxpy: y += alpha x, nothing when alpha is zero
int gsl_blas_daxpy(double alpha, const gsl_vector* x, gsl_vector* y) {
    if (x->size != y->size) GSL_ERROR("invalid length", GSL_FAILURE);
    if (alpha == 0.0) return GSL_SUCCESS;
    for (size_t i = 0; i < x->size; ++i) y->data[i] += alpha * x->data[i];
    return GSL_SUCCESS;
}

// ---- multimin fdf framework ----
gsl_multimin_fdfminimizer* gsl_multimin_fdfminimizer_alloc(const gsl_multimin_fdfminimizer_type* T, size_t n) {
    gsl_multimin_fdfminimizer* s = static_cast<gsl_multimin_fdfminimizer*>(std::calloc(1, sizeof(*s)));
    if (!s) return nullptr;
    s->x = gsl_vector_calloc(n);
    s->gradient = gsl_vector_calloc(n);
    s->dx = gsl_vector_calloc(n);
    s->state = std::malloc(T->size);
    if (!s->x || !s->gradient || !s->dx || !s->state || (T->alloc)(s->state, n) != GSL_SUCCESS) return nullptr;
    s->type = T;
    s->fdf = nullptr;
    return s;
}
int gsl_multimin_fdfminimizer_set(gsl_multimin_fdfminimizer* s, gsl_multimin_function_fdf* fdf,
                                  const gsl_vector* x, double step_size, double tol) {
    if (s->x->size != fdf->n || x->size != fdf->n) GSL_ERROR("function incompatible with solver size", GSL_FAILURE);
    s->fdf = fdf;
    gsl_vector_memcpy(s->x, x);
    gsl_vector_set_zero(s->dx);
    return (s->type->set)(s->state, s->fdf, s->x, &(s->f), s->gradient, step_size, tol);
}
int gsl_multimin_fdfminimizer_iterate(gsl_multimin_fdfminimizer* s) {
    return (s->type->iterate)(s->state, s->fdf, s->x, &(s->f), s->gradient, s->dx);
}
void gsl_multimin_fdfminimizer_free(gsl_multimin_fdfminimizer* s) {
    if (!s) return;
    (s->type->free)(s->state);
    std::free(s->state);
    gsl_vector_free(s->dx);
    gsl_vector_free(s->gradient);
    gsl_vector_free(s->x);
    std::free(s);
}

// ---- the stage loop of Solver::run on callbacks ----
extern "C" {

typedef struct {
    int32_t mode_start, mode_step, max_iterations, min_iterations, target_iterations, fd_first;
    double ftol, eps;
} ref_cfg;

typedef struct {
    double initial_metric, final_metric;
    int32_t iterations, status, n_f_evals, n_df_evals, fail_count, n_metrics;
} ref_report;

typedef double (*ref_f_fn)(const double* x, void* user);
typedef void (*ref_df_fn)(const double* x, int32_t method, int32_t mode_count, double* g, void* user);
typedef void (*ref_shift_fn)(const double* x, void* user);

// method 1: finite differences (the first gradient of a patch), 2: Vogel (solver.cpp:387, 478)
int ref_cg_minimize(int32_t n_free, int32_t n_modes, const ref_cfg* cfg, double grad_scale, ref_f_fn f,
                    ref_df_fn df, ref_shift_fn shift, void* user, double* x_out, ref_report* rep, double* metrics,
                    int32_t cap_metrics) {
    using namespace redux::util::gsl;
    if (n_free < 1 || n_modes < 1 || !cfg || !f || !df || !x_out) return -2;
    int method = cfg->fd_first ? 1 : 2;
    int modeCountNow = 0;
    int64_t nf = 0, ndf = 0;
    int32_t nMetrics = 0;
    auto push = [&](double v) {
        if (metrics && nMetrics < cap_metrics) metrics[nMetrics] = v;
        ++nMetrics;
    };
    auto my_f = [&](const gsl_vector* b, void*) -> double {
        ++nf;
        return f(b->data, user);
    };
    auto my_df = [&](const gsl_vector* b, void*, gsl_vector* g) {
        ++ndf;
        df(b->data, method, modeCountNow, g->data, user);
    };
    // Solver::my_fdf also forms a gradient, which conjugate_rdx_iterate overwrites before any
    // read (its first statement evaluates the gradient again): only the metric is requested
    auto my_fdf = [&](const gsl_vector* b, void* p, double* fv, gsl_vector*) { *fv = my_f(b, p); };
    rdx_fdf my_func(n_free, my_f, my_df, my_fdf);

    const double init_step = 1.0, init_tol = 1E-6;   // read by conjugate_rdx_set, used by nothing
    gsl_multimin_fdfminimizer* s = gsl_multimin_fdfminimizer_alloc(multimin_fdfminimizer_conjugate_rdx, n_free);
    if (!s) return -3;
    gsl_vector* beta_init = gsl_vector_calloc(n_free);
    s->f = 0;
    double previousMetric = 0, thisMetric = 0, gradNorm = 0;
    double tol = 1.0E-1;
    int failCount = 0, totalIterations = 0, maxIterations = 10;
    const int maxFails = 3;
    int status = 0;
    const double initialMetric = GSL_MULTIMIN_FN_EVAL_F(&my_func, beta_init);
    push(initialMetric);
    bool exitLoop = false;
    for (int modeCount = cfg->mode_start; !exitLoop; modeCount += cfg->mode_step) {
        modeCount = modeCount < n_modes ? modeCount : n_modes;
        modeCountNow = modeCount;
        if (modeCount == n_modes || cfg->max_iterations == 0) {
            exitLoop = true;
            tol = cfg->ftol;
            maxIterations = cfg->max_iterations;
        }
        gsl_multimin_fdfminimizer_set(s, static_cast<gsl_multimin_function_fdf*>(&my_func), beta_init, init_step,
                                      init_tol);
        int iter = 0, successCount = 0;
        bool done = false;
        while ((!done || iter < cfg->min_iterations) && iter < maxIterations) {
            iter++;
            status = gsl_multimin_fdfminimizer_iterate(s);
            if (failCount > maxFails) {
                status = GSL_FAILURE;
                exitLoop = true;
                done = true;
                break;
            }
            method = 2;
            if (status == GSL_ENOPROG) {
                failCount++;
                break;
            }
            thisMetric = s->f;
            if (!std::isfinite(thisMetric)) {
                failCount++;
                break;
            }
            push(thisMetric);
            gradNorm = gsl_blas_dnrm2(s->gradient) * grad_scale;
            if (!std::isfinite(gradNorm)) {
                failCount++;
                break;
            }
            if (gradNorm < cfg->ftol) {
                exitLoop = true;
                done = true;
                break;
            }
            if (iter > 1) {
                const double relativeChange =
                    2.0 * std::fabs(thisMetric - previousMetric) / (std::fabs(thisMetric) + std::fabs(previousMetric) + cfg->eps);
                if (relativeChange < tol) {
                    if (++successCount >= cfg->target_iterations) {
                        successCount = 0;
                        done = true;
                    }
                } else {
                    successCount = 0;
                }
            }
            previousMetric = thisMetric;
        }
        thisMetric = GSL_MULTIMIN_FN_EVAL_F(&my_func, s->x);
        totalIterations += iter;
        if (!exitLoop && shift) shift(s->x->data, user);   // shiftAndInit(); alpha_offset = alpha
    }
    std::memcpy(x_out, s->x->data, sizeof(double) * (size_t)n_free);
    if (rep) {
        rep->initial_metric = initialMetric;
        rep->final_metric = thisMetric;
        rep->iterations = totalIterations;
        rep->status = status == GSL_FAILURE ? 1 : 0;
        rep->n_f_evals = (int32_t)nf;
        rep->n_df_evals = (int32_t)ndf;
        rep->fail_count = failCount;
        rep->n_metrics = nMetrics;
    }
    gsl_vector_free(beta_init);
    gsl_multimin_fdfminimizer_free(s);
    return status == GSL_FAILURE ? 1 : 0;
}

}  // extern "C"
