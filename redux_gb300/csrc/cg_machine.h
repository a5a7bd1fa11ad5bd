// Resumable per-patch optimiser of redux's momfbd::Solver::run.
//
// The reference drives each patch with nested loops that call the metric and the
// gradient synchronously (src/lib/momfbd/solver.cpp:330-580 around GSL's
// conjugate_rdx_iterate, src/lib/util/gsl/conjugate_gradient.cpp:128-256, which in turn
// runs bracket and brent, src/lib/math/helpers.cpp:58-215).  On the GPU all patches of a
// batch advance together, one evaluation per round, so the same control flow is written
// here as an explicit state machine: advance() runs until the patch needs an evaluation
// (metric at a point, gradient at the current point, an image re-shift) and returns; the
// caller performs the evaluation for every patch at once and calls advance() again.
//
// The code is shared by the device kernel (one thread block per patch; every thread runs
// the scalar logic redundantly and the vector operations are block-parallel) and by the
// host driver rdxg_cg_minimize, so the exact sequence of evaluations can be checked on
// the CPU against the sequential restatement in the oracle.
//
// Vector storage: x (beta), p (direction), g (gradient, beta space), g0 (previous
// gradient), x1 (the point of the next evaluation) -- n_free doubles each.
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define RDXG_HD __host__ __device__
#else
#define RDXG_HD
#endif

namespace rdxg {

enum Request : int32_t {
    REQ_NONE = 0,
    REQ_F = 1,        // metric at x1
    REQ_DF = 2,       // gradient at x1 (== x); method in grad_method
    REQ_SHIFT = 3,    // re-shift the images for alpha(x1), then set alpha_offset = alpha(x1)
    REQ_DONE = 4,
};

enum GradMethod : int32_t { GM_FD = 1, GM_VOGEL = 2 };

enum Status : int32_t { ST_SUCCESS = 0, ST_ENOPROG = 27, ST_FAILURE = -1 };

struct CgParams {
    int32_t n_free;
    int32_t n_modes;
    int32_t mode_start;       // MODE_START
    int32_t mode_step;        // MODE_STEP
    int32_t max_iterations;   // MAX_ITER
    int32_t min_iterations;   // MIN_ITER
    int32_t target_iterations;// N_DONE_ITER
    int32_t fd_first;         // first gradient by finite differences (reference behaviour)
    int32_t max_fails;        // 3 in solver.cpp:404
    int32_t max_metrics;      // capacity of the metric history
    double ftol;              // FTOL
    double eps;               // EPS
    double grad_scale;        // 1 / (nTotalPixels^2)
    double brent_tol;         // 0.1
    double init_step;         // 1e-21 (initial trial step factor)
};

// program counters
enum Pc : int32_t {
    PC_START = 0,
    PC_GOT_INIT,
    PC_STAGE_BEGIN,
    PC_GOT_SET,
    PC_LOOP_TEST,
    PC_CG_START,
    PC_CG_GOT_DF,
    PC_CG_GOT_FC,
    PC_BR_START,
    PC_BR_GOT_MID,
    PC_BR_LOOP,
    PC_BR_C1,
    PC_BR_C2,
    PC_BR_SHIFT,
    PC_BR_SHIFT_NOW,
    PC_BR_END,
    PC_BT_GOT_X,
    PC_BT_LOOP,
    PC_BT_GOT_U,
    PC_CG_FINISH,
    PC_POST_ITER,
    PC_STAGE_FINISH,
    PC_STAGE_GOT_FINAL,
    PC_GOT_SHIFT,
    PC_DONE,
};

struct CgState {
    int32_t pc;
    int32_t req;             // last request issued
    int32_t grad_method;     // method for REQ_DF
    int32_t mode_count;      // number of enabled modes (first mode_count)
    int32_t exit_loop, iter, success_count, done, fail_count, total_iterations;
    int32_t max_iterations_cur, status, cg_iter, br_limit_hit;
    int32_t bt_iter, n_metrics, n_f, n_df;
    double tol, sf, previous_metric, this_metric, grad_norm, initial_metric;
    double pnorm, g0norm, g1norm, lambda;
    // bracket
    double a, b, mid, fa, fb, fmid, u, fu, ulim;
    // brent
    double bt_a, bt_b, bt_x, bt_fx, bt_v, bt_w, bt_fv, bt_fw, bt_d, bt_e, bt_u;
    double last_f;           // value delivered by the evaluator for REQ_F
};

static const double kGold = 1.6180339887498949025257;   // (1 + sqrt(5)) / 2
static const double kTiny = 1.0E-32;

RDXG_HD inline double sgn_abs(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

// V must provide (collective on the device):
//   void   copy(double* dst, const double* src);             n_free
//   void   zero(double* dst);
//   double nrm2(const double* v);
//   double dot(const double* a, const double* b);
//   double pr_update(double* g0, const double* g);           g0 <- g0 - g, returns (g0-g).g
//   void   dir_update(double* p, const double* g, double beta);  p <- g - beta p
//   void   step(double* x1, const double* x, const double* p, double s);  x1 <- x + s p
//   void   sync();                                            barrier after scalar writes
template <class V>
struct Machine {
    const CgParams& P;
    CgState& S;
    V& v;
    double *x, *p, *g, *g0, *x1;
    double* metrics;   // history (may be null)

    RDXG_HD Machine(const CgParams& prm, CgState& st, V& vops, double* x_, double* p_, double* g_,
                    double* g0_, double* x1_, double* metrics_)
        : P(prm), S(st), v(vops), x(x_), p(p_), g(g_), g0(g0_), x1(x1_), metrics(metrics_) {}

    RDXG_HD void push_metric(double m) {
        if (metrics && S.n_metrics < P.max_metrics) metrics[S.n_metrics] = m;
        S.n_metrics++;
    }

    // take_step (conjugate_gradient.cpp:106-113): x1 = x + (-s*lambda) p
    RDXG_HD void request_at_step(double s) {
        v.step(x1, x, p, -s * S.lambda);
        S.req = REQ_F;
    }
    RDXG_HD void request_at_x() {
        v.copy(x1, x);
        S.req = REQ_F;
    }

    // Runs until a request is issued; returns the request.  `f` is the value of the last
    // REQ_F evaluation (ignored otherwise).
    RDXG_HD int32_t advance(double f) {
        S.last_f = f;
        S.req = REQ_NONE;
        for (;;) {
            switch (S.pc) {
            case PC_START: {
                S.mode_count = 0;
                S.exit_loop = 0; S.fail_count = 0; S.total_iterations = 0;
                S.max_iterations_cur = 10; S.status = ST_SUCCESS;
                S.tol = 1.0E-1; S.previous_metric = 0; S.this_metric = 0; S.grad_norm = 0;
                S.n_metrics = 0; S.n_f = 0; S.n_df = 0; S.br_limit_hit = 0;
                S.grad_method = P.fd_first ? GM_FD : GM_VOGEL;
                S.cg_iter = 0; S.pnorm = 0; S.g0norm = 0;
                v.zero(x);
                request_at_x();                  // initialMetric = f(beta_init = 0)
                S.pc = PC_GOT_INIT;
                S.n_f++;
                return S.req;
            }
            case PC_GOT_INIT:
                S.initial_metric = S.last_f;
                push_metric(S.last_f);
                S.mode_count = P.mode_start;
                S.pc = PC_STAGE_BEGIN;
                break;
            case PC_STAGE_BEGIN: {
                if (S.mode_count > P.n_modes) S.mode_count = P.n_modes;
                if (S.mode_count == P.n_modes || P.max_iterations == 0) {
                    S.exit_loop = 1;
                    S.tol = P.ftol;
                    S.max_iterations_cur = P.max_iterations;
                }
                // gsl_multimin_fdfminimizer_set: x = beta_init (0); conjugate_rdx_set evaluates
                // f and a gradient; the gradient is overwritten by the first iterate before it
                // is read, so only f is requested.
                v.zero(x);
                S.cg_iter = 0;
                request_at_x();
                S.pc = PC_GOT_SET;
                S.n_f++;
                return S.req;
            }
            case PC_GOT_SET:
                S.sf = S.last_f;
                S.iter = 0; S.success_count = 0; S.done = 0;
                S.pc = PC_LOOP_TEST;
                break;
            case PC_LOOP_TEST:
                if (!((!S.done || S.iter < P.min_iterations) && S.iter < S.max_iterations_cur)) {
                    S.pc = PC_STAGE_FINISH;
                    break;
                }
                S.iter++;
                S.pc = PC_CG_START;
                break;
            case PC_CG_START:
                // conjugate_rdx_iterate: gradient at x
                v.copy(x1, x);
                S.req = REQ_DF;
                S.pc = PC_CG_GOT_DF;
                S.n_df++;
                return S.req;
            case PC_CG_GOT_DF: {
                double pg;
                S.g1norm = v.nrm2(g);
                if (S.cg_iter++ == 0) {
                    v.copy(p, g);
                    S.pnorm = S.g1norm;
                    pg = S.g1norm * S.g1norm;
                } else {
                    if (S.g0norm == 0.0) {
                        S.status = ST_ENOPROG;
                        S.pc = PC_POST_ITER;
                        break;
                    }
                    double g0g1 = v.pr_update(g0, g);
                    double beta = g0g1 / (S.g0norm * S.g0norm);
                    v.dir_update(p, g, beta);
                    S.pnorm = v.nrm2(p);
                    pg = v.dot(p, g);
                }
                S.lambda = (pg >= 0.0) ? +1.0 / S.pnorm : -1.0 / S.pnorm;
                if (S.pnorm == 0.0) {
                    S.status = ST_ENOPROG;
                    S.pc = PC_POST_ITER;
                    break;
                }
                S.fa = S.sf;
                S.a = 0.0;
                S.b = P.init_step / S.lambda;     // stepc = 1E-21/lambda
                request_at_step(S.b);
                S.pc = PC_CG_GOT_FC;
                S.n_f++;
                return S.req;
            }
            case PC_CG_GOT_FC:
                S.fb = S.last_f;                   // fc
                S.pc = PC_BR_START;
                break;
            // ---------------- bracket (helpers.cpp:58-129) ----------------
            case PC_BR_START:
                if (S.fb > S.fa) {
                    double t = S.a; S.a = S.b; S.b = t;
                    t = S.fa; S.fa = S.fb; S.fb = t;
                }
                S.mid = S.b + kGold * (S.b - S.a);
                request_at_step(S.mid);
                S.pc = PC_BR_GOT_MID;
                S.n_f++;
                return S.req;
            case PC_BR_GOT_MID:
                S.fmid = S.last_f;
                S.pc = PC_BR_LOOP;
                break;
            case PC_BR_LOOP: {
                if (!(S.fb > S.fmid)) { S.pc = PC_BR_END; break; }
                const double r = (S.b - S.a) * (S.fb - S.fmid);
                const double q = (S.b - S.mid) * (S.fb - S.fa);
                const double mx = fabs(q - r) > kTiny ? fabs(q - r) : kTiny;
                S.u = S.b - ((S.b - S.mid) * q - (S.b - S.a) * r) / (2.0 * sgn_abs(mx, q - r));
                S.ulim = S.b + 100 * (S.mid - S.b);
                if ((S.b - S.u) * (S.u - S.mid) > 0.0) {
                    request_at_step(S.u);
                    S.pc = PC_BR_C1;
                } else if ((S.mid - S.u) * (S.u - S.ulim) > 0.0) {
                    request_at_step(S.u);
                    S.pc = PC_BR_C2;
                } else if ((S.mid - S.ulim) * (S.ulim - S.u) >= 0.0) {
                    S.u = S.ulim;
                    request_at_step(S.u);
                    S.pc = PC_BR_SHIFT;
                } else {
                    S.u = S.mid + kGold * (S.mid - S.b);
                    request_at_step(S.u);
                    S.pc = PC_BR_SHIFT;
                }
                S.n_f++;
                return S.req;
            }
            case PC_BR_C1:
                S.fu = S.last_f;
                if (S.fu < S.fmid) {
                    S.a = S.b; S.b = S.u; S.fa = S.fb; S.fb = S.fu;
                    S.pc = PC_BR_END;
                    break;
                } else if (S.fu > S.fb) {
                    S.mid = S.u; S.fmid = S.fu;
                    S.pc = PC_BR_END;
                    break;
                }
                S.u = S.mid + kGold * (S.mid - S.b);
                request_at_step(S.u);
                S.pc = PC_BR_SHIFT;
                S.n_f++;
                return S.req;
            case PC_BR_C2:
                S.fu = S.last_f;
                if (S.fu < S.fmid) {
                    S.b = S.mid; S.mid = S.u; S.u = S.mid + kGold * (S.mid - S.b);
                    S.fb = S.fmid; S.fmid = S.fu;
                    request_at_step(S.u);
                    S.pc = PC_BR_SHIFT;
                    S.n_f++;
                    return S.req;
                }
                S.pc = PC_BR_SHIFT_NOW;
                break;
            case PC_BR_SHIFT:
                S.fu = S.last_f;
                S.pc = PC_BR_SHIFT_NOW;
                break;
            case PC_BR_SHIFT_NOW:
                S.a = S.b; S.b = S.mid; S.mid = S.u;
                S.fa = S.fb; S.fb = S.fmid; S.fmid = S.fu;
                S.pc = PC_BR_LOOP;
                break;
            case PC_BR_END: {
                if (S.a > S.b) { double t = S.a; S.a = S.b; S.b = t; t = S.fa; S.fa = S.fb; S.fb = t; }
                if (S.mid > S.b) { double t = S.mid; S.mid = S.b; S.b = t; t = S.fmid; S.fmid = S.fb; S.fb = t; }
                if (S.mid < S.a) { double t = S.mid; S.mid = S.a; S.a = t; t = S.fmid; S.fmid = S.fa; S.fa = t; }
                // brent(value_at, stepa=a, stepc=b, stepb=mid, fb=fmid, tol)
                S.bt_a = S.a < S.b ? S.a : S.b;
                S.bt_b = S.a > S.b ? S.a : S.b;
                S.bt_x = S.mid;
                S.bt_u = S.bt_v = S.bt_w = S.bt_x;
                request_at_step(S.bt_x);
                S.pc = PC_BT_GOT_X;
                S.n_f++;
                return S.req;
            }
            // ---------------- brent (helpers.cpp:133-215) ----------------
            case PC_BT_GOT_X:
                S.fu = S.bt_fv = S.bt_fw = S.bt_fx = S.last_f;
                S.bt_d = 0.0; S.bt_e = 0.0;
                S.bt_iter = 1;
                S.pc = PC_BT_LOOP;
                break;
            case PC_BT_LOOP: {
                if (S.bt_iter > 100) {
                    S.br_limit_hit++;      // "Error in brent: too many iterations!"
                    S.pc = PC_CG_FINISH;
                    break;
                }
                const double xm = 0.5 * (S.bt_a + S.bt_b);
                const double tol1 = P.brent_tol * fabs(S.bt_x) + kTiny;
                const double tol2 = 2.0 * tol1;
                if (fabs(S.bt_x - xm) <= (tol2 - 0.5 * (S.bt_b - S.bt_a))) {
                    S.pc = PC_CG_FINISH;
                    break;
                }
                const double CGOLD = 2.0 - kGold;
                if (fabs(S.bt_e) > tol1) {
                    double r = (S.bt_x - S.bt_w) * (S.bt_fx - S.bt_fv);
                    double q = (S.bt_x - S.bt_v) * (S.bt_fx - S.bt_fw);
                    double pp = (S.bt_x - S.bt_v) * q - (S.bt_x - S.bt_w) * r;
                    q = 2.0 * (q - r);
                    if (q > 0.0) pp = -pp;
                    q = fabs(q);
                    double etemp = S.bt_e;
                    S.bt_e = S.bt_d;
                    if (fabs(pp) >= fabs(0.5 * q * etemp) || pp <= q * (S.bt_a - S.bt_x) ||
                        pp >= q * (S.bt_b - S.bt_x)) {
                        S.bt_e = (S.bt_x >= xm ? S.bt_a - S.bt_x : S.bt_b - S.bt_x);
                        S.bt_d = CGOLD * S.bt_e;
                    } else {
                        S.bt_d = pp / q;
                        S.bt_u = S.bt_x + S.bt_d;
                        if (S.bt_u - S.bt_a < tol2 || S.bt_b - S.bt_u < tol2) S.bt_d = sgn_abs(tol1, xm - S.bt_x);
                    }
                } else {
                    S.bt_e = (S.bt_x >= xm ? S.bt_a - S.bt_x : S.bt_b - S.bt_x);
                    S.bt_d = CGOLD * S.bt_e;
                }
                if (fabs(S.bt_d) < tol1) S.bt_d *= (tol1 / fabs(S.bt_d));
                S.bt_u = ((fabs(S.bt_d) >= tol1) ? S.bt_x + S.bt_d : S.bt_x + sgn_abs(tol1, S.bt_d));
                request_at_step(S.bt_u);
                S.pc = PC_BT_GOT_U;
                S.n_f++;
                return S.req;
            }
            case PC_BT_GOT_U: {
                const double fu = S.last_f;
                if (fu <= S.bt_fx) {
                    if (S.bt_u >= S.bt_x) S.bt_a = S.bt_x; else S.bt_b = S.bt_x;
                    S.bt_v = S.bt_w; S.bt_w = S.bt_x; S.bt_x = S.bt_u;
                    S.bt_fv = S.bt_fw; S.bt_fw = S.bt_fx; S.bt_fx = fu;
                } else {
                    if (S.bt_u < S.bt_x) S.bt_a = S.bt_u; else S.bt_b = S.bt_u;
                    if (fu <= S.bt_fw || S.bt_w == S.bt_x) {
                        S.bt_v = S.bt_w; S.bt_w = S.bt_u; S.bt_fv = S.bt_fw; S.bt_fw = fu;
                    } else if (fu <= S.bt_fv || S.bt_v == S.bt_x || S.bt_v == S.bt_w) {
                        S.bt_v = S.bt_u; S.bt_fv = fu;
                    }
                }
                S.bt_iter++;
                S.pc = PC_BT_LOOP;
                break;
            }
            case PC_CG_FINISH: {
                // move to the line minimum (conjugate_gradient.cpp:240-252)
                v.step(x1, x, p, -S.bt_x * S.lambda);
                v.copy(x, x1);
                S.sf = S.bt_fx;
                S.g0norm = S.g1norm;
                v.copy(g0, g);
                S.cg_iter = S.cg_iter % P.n_free;
                S.status = ST_SUCCESS;
                S.pc = PC_POST_ITER;
                break;
            }
            // ---------------- Solver::run inner loop checks (solver.cpp:469-517) ----------------
            case PC_POST_ITER: {
                if (S.fail_count > P.max_fails) {
                    S.status = ST_FAILURE;
                    S.exit_loop = 1; S.done = 1;
                    S.pc = PC_STAGE_FINISH;
                    break;
                }
                S.grad_method = GM_VOGEL;
                if (S.status == ST_ENOPROG) { S.fail_count++; S.pc = PC_STAGE_FINISH; break; }
                S.this_metric = S.sf;
                if (!isfinite(S.this_metric)) { S.fail_count++; S.pc = PC_STAGE_FINISH; break; }
                push_metric(S.this_metric);
                S.grad_norm = v.nrm2(g) * P.grad_scale;
                if (!isfinite(S.grad_norm)) { S.fail_count++; S.pc = PC_STAGE_FINISH; break; }
                if (S.grad_norm < P.ftol) {
                    S.exit_loop = 1; S.done = 1;
                    S.pc = PC_STAGE_FINISH;
                    break;
                }
                if (S.iter > 1) {
                    double rc = 2.0 * fabs(S.this_metric - S.previous_metric) /
                                (fabs(S.this_metric) + fabs(S.previous_metric) + P.eps);
                    if (rc < S.tol) {
                        if (++S.success_count >= P.target_iterations) { S.success_count = 0; S.done = 1; }
                    } else {
                        S.success_count = 0;
                    }
                }
                S.previous_metric = S.this_metric;
                S.pc = PC_LOOP_TEST;
                break;
            }
            case PC_STAGE_FINISH:
                request_at_x();
                S.pc = PC_STAGE_GOT_FINAL;
                S.n_f++;
                return S.req;
            case PC_STAGE_GOT_FINAL:
                S.this_metric = S.last_f;
                S.total_iterations += S.iter;
                if (!S.exit_loop) {
                    // shiftAndInit(); alpha_offset = alpha  -- x1 still holds x
                    S.req = REQ_SHIFT;
                    S.pc = PC_GOT_SHIFT;
                    return S.req;
                }
                S.pc = PC_DONE;
                break;
            case PC_GOT_SHIFT:
                S.mode_count += P.mode_step;
                S.pc = PC_STAGE_BEGIN;
                break;
            case PC_DONE:
            default:
                S.req = REQ_DONE;
                S.pc = PC_DONE;
                return S.req;
            }
        }
    }
};

}  // namespace rdxg
