/*
 * oracle.c -- FP64 CPU restatement of redux's per-patch MOMFBD solver.
 *
 * TEST INFRASTRUCTURE ONLY.  The GPU solver in redux_gb300 is tested against this
 * restatement: only tests/, __graft_entry__.smoke() and bench.py's CPU baseline leg may
 * load it.  The product never links, imports or calls it.
 *
 * It restates, in plain C99 and double precision, the reference code of the
 * MOMFBD hot path (paths relative to the ISP-SST/redux tree):
 *   src/lib/momfbd/subimage.cpp    getWindowedImg 106-150, initialize 155-209,
 *                                  addPQ 226-234, metricChange 261-278,
 *                                  gradientFiniteDifference 281-292,
 *                                  gradientVogel 312-326, calcVogelWeight 348-390,
 *                                  adjustShifts 444-480, addToPhi/calcPhi 509-544,
 *                                  calcOTF 567-583, calcPFOTF 586-612
 *   src/lib/momfbd/object.cpp      initPQ 459, addRegGamma 465, addToFT 471,
 *                                  addDiffToFT 482, addToPQ 508, calcHelpers 531,
 *                                  calcMetric 597-615, reInitialize 885-904
 *   src/lib/momfbd/solver.cpp      run 330-580, applyBeta 662, metric 763-817,
 *                                  calcPQ 820-857, gradient 860-902
 *   src/lib/momfbd/channel.cpp     initPatch (phi_channel, otfNormalization) 846-953
 *   include/redux/momfbd/constraints.hpp  apply/reverse/reverseAndAdd 128-159
 *   src/lib/util/gsl/conjugate_gradient.cpp  conjugate_rdx_set 72-86,
 *                                  take_step/value_at 106-123, iterate 128-256
 *   src/lib/math/helpers.cpp       bracket 58-129, brent 133-215
 *   src/lib/image/fouriertransform.cpp  noise 448-495; fouriertransform.hpp
 *                                  reorderInto 112-171, autocorrelate 281-286
 *
 * Third-party arithmetic: the reference transforms with FFTW3 (unpinned
 * version; fftw_plan_dft_2d, FFTW_MEASURE).  FFTW computes the plain DFT
 * X[k] = sum_x x[x] exp(-2 pi i k.x/N) (forward) and the unnormalised inverse
 * with exp(+...); this file implements the same DFT with its own mixed-radix
 * recursive FFT, pinned by the known-answer tests of
 * testsuite/image/fourier.cpp restated in tests/test_oracle_fft.py.
 *
 * Parity status: the FFT/autocorrelation/reorder conventions are pinned by the
 * reference's known-answer tests.  The conjugate-gradient iteration, bracket and
 * brent (and the Solver::run stage loop around them, orc_cg_minimize) are pinned
 * bit for bit against the reference's own conjugate_gradient.cpp and helpers.cpp
 * compiled from its sources into oracle/_ref (tests/test_ref_minimizer.py).  The
 * reference has no tests for the metric or gradient and the rest of it cannot be
 * built here (Boost, FFTW3, GSL and OpenCV are absent), so those parts are
 * "parity unpinned": they follow the cited source line by line and are
 * cross-checked against an independent numpy restatement (oracle/np_oracle.py)
 * and against finite differences.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* ------------------------------------------------------------------------- */
/* FFT: recursive mixed-radix decimation in time (any length).               */
/* ------------------------------------------------------------------------- */

typedef struct {
    int n;
    int nfac;
    int fac[40];
    cplx* tw_fwd; /* exp(-2 pi i k / n), k < n */
    cplx* tw_bwd; /* exp(+2 pi i k / n) */
    /* iterative form (fft1_fast): its own factorisation (radix 8 first, then 4, 2 and the odd
     * primes); per stage s, twiddles exp(-+2 pi i r k / (NS R)) for k < NS, r < R
     * (interleaved cos, sin), NS = product of the earlier radices; cos and sin of 2 pi q / R
     * for each odd radix */
    int nffac;
    int ffac[40];
    double* st_tw[2];
    int st_off[41];
    double* odd_cs;
    int odd_off[40];
} fft_plan;

/* Which transform the solver's FFTs use: 0 the recursive one above (the oracle proper), 1 the
 * iterative Stockham form with precomputed tables, real arithmetic and stages specialised per
 * radix (orc_set_fast_fft; used to time the CPU baseline: the same DFT, factorised with radix 8
 * first and rounded differently). */
static int g_fast_fft = 0;
void orc_set_fast_fft(int on) { g_fast_fft = on ? 1 : 0; }
static void plan_fast_init(fft_plan* p);

static void plan_init(fft_plan* p, int n) {
    p->n = n;
    p->nfac = 0;
    int m = n;
    /* radix-4 first (fewer stages), then 2, 3, 5, ..., any prime */
    while (m % 4 == 0) { p->fac[p->nfac++] = 4; m /= 4; }
    while (m % 2 == 0) { p->fac[p->nfac++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2) {
        while (m % f == 0) { p->fac[p->nfac++] = f; m /= f; }
    }
    p->tw_fwd = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    p->tw_bwd = (cplx*)malloc(sizeof(cplx) * (size_t)n);
    for (int k = 0; k < n; ++k) {
        double a = 2.0 * M_PI * (double)k / (double)n;
        p->tw_fwd[k] = cos(a) - I * sin(a);
        p->tw_bwd[k] = cos(a) + I * sin(a);
    }
    plan_fast_init(p);
}

static void plan_fast_init(fft_plan* p) {
    const int n = p->n;
    p->nffac = 0;
    int m = n;
    while (m % 8 == 0) { p->ffac[p->nffac++] = 8; m /= 8; }
    while (m % 4 == 0) { p->ffac[p->nffac++] = 4; m /= 4; }
    while (m % 2 == 0) { p->ffac[p->nffac++] = 2; m /= 2; }
    for (int f = 3; m > 1; f += 2) {
        while (m % f == 0) { p->ffac[p->nffac++] = f; m /= f; }
    }
    int tot = 0, ns = 1, nodd = 0;
    for (int s = 0; s < p->nffac; ++s) {
        p->st_off[s] = tot;
        tot += ns * p->ffac[s];
        ns *= p->ffac[s];
        p->odd_off[s] = nodd;
        if (p->ffac[s] % 2) nodd += p->ffac[s];
    }
    p->st_off[p->nffac] = tot;
    for (int d = 0; d < 2; ++d) p->st_tw[d] = (double*)malloc(sizeof(double) * 2 * (size_t)(tot > 0 ? tot : 1));
    p->odd_cs = (double*)malloc(sizeof(double) * 2 * (size_t)(nodd > 0 ? nodd : 1));
    ns = 1;
    for (int s = 0; s < p->nffac; ++s) {
        const int R = p->ffac[s];
        for (int k = 0; k < ns; ++k)
            for (int r = 0; r < R; ++r) {
                const double a = 2.0 * M_PI * (double)r * (double)k / (double)(ns * R);
                const int o = 2 * (p->st_off[s] + k * R + r);
                p->st_tw[0][o] = cos(a); p->st_tw[0][o + 1] = -sin(a);
                p->st_tw[1][o] = cos(a); p->st_tw[1][o + 1] = sin(a);
            }
        if (R % 2)
            for (int q = 0; q < R; ++q) {
                p->odd_cs[2 * (p->odd_off[s] + q)] = cos(2.0 * M_PI * q / R);
                p->odd_cs[2 * (p->odd_off[s] + q) + 1] = sin(2.0 * M_PI * q / R);
            }
        ns *= R;
    }
    (void)n;
}

static void plan_free(fft_plan* p) {
    free(p->tw_fwd);
    free(p->tw_bwd);
    free(p->st_tw[0]);
    free(p->st_tw[1]);
    free(p->odd_cs);
    p->tw_fwd = p->tw_bwd = NULL;
    p->st_tw[0] = p->st_tw[1] = NULL;
    p->odd_cs = NULL;
}

/* out[0..L) = DFT_L of in[q*istride]; fi = index into p->fac; L = prod fac[fi..] */
static void fft_rec(const fft_plan* p, const cplx* tw, cplx* out, const cplx* in, long istride,
                    int fi, long L, long fstride) {
    int r = p->fac[fi];
    long m = L / r;
    if (m == 1) {
        for (int q = 0; q < r; ++q) out[q] = in[q * istride];
    } else {
        for (int q = 0; q < r; ++q)
            fft_rec(p, tw, out + q * m, in + q * istride, istride * r, fi + 1, m, fstride * r);
    }
    const int N = p->n;
    cplx t[64];
    cplx* tt = (r <= 64) ? t : (cplx*)malloc(sizeof(cplx) * (size_t)r);
    for (long k = 0; k < m; ++k) {
        for (int q = 0; q < r; ++q) {
            long e = ((long)q * k * fstride) % N;
            tt[q] = out[q * m + k] * tw[e];
        }
        if (r == 2) {
            out[k] = tt[0] + tt[1];
            out[k + m] = tt[0] - tt[1];
        } else if (r == 4) {
            /* w = exp(sign 2 pi i / 4): sign taken from tw[N/4] */
            cplx w = tw[N / 4];
            cplx a0 = tt[0] + tt[2], a1 = tt[0] - tt[2];
            cplx b0 = tt[1] + tt[3], b1 = (tt[1] - tt[3]) * w;
            out[k] = a0 + b0;
            out[k + m] = a1 + b1;
            out[k + 2 * m] = a0 - b0;
            out[k + 3 * m] = a1 - b1;
        } else {
            long step = N / r;
            for (int u = 0; u < r; ++u) {
                cplx s = 0;
                for (int q = 0; q < r; ++q) s += tt[q] * tw[((long)q * u * step) % N];
                out[k + u * m] = s;
            }
        }
    }
    if (tt != t) free(tt);
}

/* One stage of the iterative Stockham transform below: radix R (a compile-time constant at
 * each call, so that the loops over the butterfly's R values unroll), NS = product of the
 * earlier radices; a -> b. */
static inline __attribute__((always_inline)) void fast_stage(const fft_plan* p, int s, const double* a, double* b,
                                                             int ns, const int R, double dsg, const double* tws) {
    const int n = p->n;
    const int bf = n / R;
    const double* tw = tws + 2 * p->st_off[s];
    const double* cs = (R % 2) ? p->odd_cs + 2 * p->odd_off[s] : NULL;
    double vr[64], vi[64];
    for (int j = 0; j < bf; ++j) {
        const int k = j % ns;
        for (int r = 0; r < R; ++r) {
            vr[r] = a[2 * (j + r * bf)];
            vi[r] = a[2 * (j + r * bf) + 1];
        }
        if (ns > 1) {
            const double* w = tw + 2 * k * R;
            for (int r = 1; r < R; ++r) {
                const double xr = vr[r], xi = vi[r];
                vr[r] = xr * w[2 * r] - xi * w[2 * r + 1];
                vi[r] = xr * w[2 * r + 1] + xi * w[2 * r];
            }
        }
        const int d0 = (j / ns) * ns * R + k;
        if (R == 2) {
            b[2 * d0] = vr[0] + vr[1]; b[2 * d0 + 1] = vi[0] + vi[1];
            b[2 * (d0 + ns)] = vr[0] - vr[1]; b[2 * (d0 + ns) + 1] = vi[0] - vi[1];
        } else if (R == 4) {
            const double a0r = vr[0] + vr[2], a0i = vi[0] + vi[2], a1r = vr[0] - vr[2], a1i = vi[0] - vi[2];
            const double b0r = vr[1] + vr[3], b0i = vi[1] + vi[3];
            /* (v1 - v3) * i sign */
            const double tr = vr[1] - vr[3], ti = vi[1] - vi[3];
            const double b1r = -dsg * ti, b1i = dsg * tr;
            b[2 * d0] = a0r + b0r; b[2 * d0 + 1] = a0i + b0i;
            b[2 * (d0 + ns)] = a1r + b1r; b[2 * (d0 + ns) + 1] = a1i + b1i;
            b[2 * (d0 + 2 * ns)] = a0r - b0r; b[2 * (d0 + 2 * ns) + 1] = a0i - b0i;
            b[2 * (d0 + 3 * ns)] = a1r - b1r; b[2 * (d0 + 3 * ns) + 1] = a1i - b1i;
        } else if (R == 8) {
            /* y[u] = E[u mod 4] + w^u O[u mod 4], w = exp(sign 2 pi i / 8): E, O the 4-point
             * transforms of the even and odd inputs */
            double er[4], ei[4], orr[4], oi[4];
            for (int h = 0; h < 2; ++h) {
                double* xr = h ? orr : er;
                double* xi = h ? oi : ei;
                const double a0r = vr[h] + vr[h + 4], a0i = vi[h] + vi[h + 4];
                const double a1r = vr[h] - vr[h + 4], a1i = vi[h] - vi[h + 4];
                const double b0r = vr[h + 2] + vr[h + 6], b0i = vi[h + 2] + vi[h + 6];
                const double tr = vr[h + 2] - vr[h + 6], ti = vi[h + 2] - vi[h + 6];
                const double b1r = -dsg * ti, b1i = dsg * tr;
                xr[0] = a0r + b0r; xi[0] = a0i + b0i;
                xr[1] = a1r + b1r; xi[1] = a1i + b1i;
                xr[2] = a0r - b0r; xi[2] = a0i - b0i;
                xr[3] = a1r - b1r; xi[3] = a1i - b1i;
            }
            const double hh = 0.70710678118654752440;   /* sqrt(1/2) */
            const double t1r = hh * (orr[1] - dsg * oi[1]), t1i = hh * (oi[1] + dsg * orr[1]);
            const double t2r = -dsg * oi[2], t2i = dsg * orr[2];
            const double t3r = hh * (-orr[3] - dsg * oi[3]), t3i = hh * (-oi[3] + dsg * orr[3]);
            const double tr_[4] = {orr[0], t1r, t2r, t3r}, ti_[4] = {oi[0], t1i, t2i, t3i};
            for (int u = 0; u < 4; ++u) {
                b[2 * (d0 + u * ns)] = er[u] + tr_[u]; b[2 * (d0 + u * ns) + 1] = ei[u] + ti_[u];
                b[2 * (d0 + (u + 4) * ns)] = er[u] - tr_[u]; b[2 * (d0 + (u + 4) * ns) + 1] = ei[u] - ti_[u];
            }
        } else {
            /* odd radix: pair x[q] with x[R-q] */
            const int H = (R - 1) / 2;
            double ar[32], ai[32], br[32], bi[32];
            double y0r = vr[0], y0i = vi[0];
            for (int q = 1; q <= H; ++q) {
                ar[q] = vr[q] + vr[R - q]; ai[q] = vi[q] + vi[R - q];
                br[q] = vr[q] - vr[R - q]; bi[q] = vi[q] - vi[R - q];
                y0r += ar[q]; y0i += ai[q];
            }
            b[2 * d0] = y0r; b[2 * d0 + 1] = y0i;
            for (int u = 1; u <= H; ++u) {
                double Ar = vr[0], Ai = vi[0], Br = 0, Bi = 0;
                int kk = 0;   /* (q * u) mod R, stepped without a division */
                for (int q = 1; q <= H; ++q) {
                    kk += u;
                    if (kk >= R) kk -= R;
                    Ar += ar[q] * cs[2 * kk]; Ai += ai[q] * cs[2 * kk];
                    Br += br[q] * cs[2 * kk + 1]; Bi += bi[q] * cs[2 * kk + 1];
                }
                /* y[u] = A + i sign B, y[R-u] = A - i sign B */
                const double ibr = -dsg * Bi, ibi = dsg * Br;
                b[2 * (d0 + u * ns)] = Ar + ibr; b[2 * (d0 + u * ns) + 1] = Ai + ibi;
                b[2 * (d0 + (R - u) * ns)] = Ar - ibr; b[2 * (d0 + (R - u) * ns) + 1] = Ai - ibi;
            }
        }
    }
}

/* Iterative Stockham transform of the n values in a (interleaved re, im); b is scratch of the
 * same size.  Returns the buffer holding the result. */
static double* fft1_fast_core(const fft_plan* p, double* a, double* b, int sign) {
    const double* tws = p->st_tw[sign < 0 ? 0 : 1];
    const double dsg = sign < 0 ? -1.0 : 1.0;
    int ns = 1;
    for (int s = 0; s < p->nffac; ++s) {
        const int R = p->ffac[s];
        switch (R) {
            case 2: fast_stage(p, s, a, b, ns, 2, dsg, tws); break;
            case 3: fast_stage(p, s, a, b, ns, 3, dsg, tws); break;
            case 4: fast_stage(p, s, a, b, ns, 4, dsg, tws); break;
            case 8: fast_stage(p, s, a, b, ns, 8, dsg, tws); break;
            case 5: fast_stage(p, s, a, b, ns, 5, dsg, tws); break;
            case 7: fast_stage(p, s, a, b, ns, 7, dsg, tws); break;
            case 11: fast_stage(p, s, a, b, ns, 11, dsg, tws); break;
            case 13: fast_stage(p, s, a, b, ns, 13, dsg, tws); break;
            default: fast_stage(p, s, a, b, ns, R, dsg, tws); break;
        }
        double* t = a; a = b; b = t;
        ns *= R;
    }
    return a;
}

/* in-place 1-D transform of x[0..n) with stride; sign<0 forward (FFTW_FORWARD) */
static void fft1(const fft_plan* p, cplx* x, long stride, int sign, cplx* work, cplx* work2) {
    const int n = p->n;
    if (g_fast_fft && p->nffac > 0) {
        int ok = 1;
        for (int s = 0; s < p->nffac; ++s)
            if (p->ffac[s] > 63) ok = 0;
        if (ok) {
            if (stride == 1) {
                /* a contiguous line is already interleaved (re, im): transform it in place, the
                 * scratch taking every other stage */
                double* xa = (double*)x;
                const double* r = fft1_fast_core(p, xa, (double*)work, sign);
                if (r != xa) memcpy(xa, r, sizeof(double) * 2 * (size_t)n);
                return;
            }
            double* a = (double*)work;
            for (int i = 0; i < n; ++i) { a[2 * i] = creal(x[i * stride]); a[2 * i + 1] = cimag(x[i * stride]); }
            const double* r = fft1_fast_core(p, a, (double*)work2, sign);
            for (int i = 0; i < n; ++i) x[i * stride] = r[2 * i] + I * r[2 * i + 1];
            return;
        }
    }
    for (int i = 0; i < n; ++i) work[i] = x[i * stride];
    fft_rec(p, sign < 0 ? p->tw_fwd : p->tw_bwd, work2, work, 1, 0, n, 1);
    for (int i = 0; i < n; ++i) x[i * stride] = work2[i];
}

/* unnormalised 2-D transform of a ny x nx row-major array */
static void fft2(const fft_plan* py, const fft_plan* px, cplx* a, int sign, cplx* work) {
    const int ny = py->n, nx = px->n;
    int mx = ny > nx ? ny : nx;
    cplx* w1 = work;
    cplx* w2 = work + mx;
    for (int y = 0; y < ny; ++y) fft1(px, a + (long)y * nx, 1, sign, w1, w2);
    for (int x = 0; x < nx; ++x) fft1(py, a + x, nx, sign, w1, w2);
}

/* reorderInto for even and odd sizes, same size in/out (fouriertransform.hpp:112-171,
 * center=false, outSize==inSize): a quadrant swap, i.e. fftshift for even sizes. */
static void reorder_c(cplx* a, int ny, int nx, cplx* buf) {
    const int midY = ny / 2, midX = nx / 2, oddY = ny % 2, oddX = nx % 2;
    /* out[(y + ny - midY - oddY) % ny][(x + nx - midX - oddX) % nx] = in[y][x] for the
     * quadrant layout used by reorderInto: the lower block is one pixel larger for odd sizes. */
    for (int y = 0; y < ny; ++y) {
        int oy = (y + midY) % ny;  /* in row y goes to out row (y + midY) mod ny */
        for (int x = 0; x < nx; ++x) {
            int ox = (x + midX) % nx;
            buf[(long)oy * nx + ox] = a[(long)y * nx + x];
        }
    }
    (void)oddY; (void)oddX;
    memcpy(a, buf, sizeof(cplx) * (size_t)ny * nx);
}

static void reorder_d(double* a, int ny, int nx, double* buf) {
    const int midY = ny / 2, midX = nx / 2;
    for (int y = 0; y < ny; ++y) {
        int oy = (y + midY) % ny;
        for (int x = 0; x < nx; ++x) {
            int ox = (x + midX) % nx;
            buf[(long)oy * nx + ox] = a[(long)y * nx + x];
        }
    }
    memcpy(a, buf, sizeof(double) * (size_t)ny * nx);
}

/* ------------------------------------------------------------------------- */
/* Exported FFT helpers, used by the known-answer tests.                     */
/* ------------------------------------------------------------------------- */

/* data: interleaved complex, ny x nx; sign -1 forward, +1 backward (unnormalised) */
void orc_fft2(double* data, int ny, int nx, int sign) {
    fft_plan py, px;
    plan_init(&py, ny);
    plan_init(&px, nx);
    int mx = ny > nx ? ny : nx;
    cplx* work = (cplx*)malloc(sizeof(cplx) * 2 * (size_t)mx);
    fft2(&py, &px, (cplx*)data, sign, work);
    free(work);
    plan_free(&py);
    plan_free(&px);
}

void orc_reorder(double* data, int ny, int nx, int is_complex) {
    if (is_complex) {
        cplx* buf = (cplx*)malloc(sizeof(cplx) * (size_t)ny * nx);
        reorder_c((cplx*)data, ny, nx, buf);
        free(buf);
    } else {
        double* buf = (double*)malloc(sizeof(double) * (size_t)ny * nx);
        reorder_d(data, ny, nx, buf);
        free(buf);
    }
}

/* FourierTransform::autocorrelate(in, out, center) (fouriertransform.hpp:281-286) for
 * real input: ft (FULLCOMPLEX) -> |.|^2 -> ift normalised by 1/(ny*nx) -> real part ->
 * optional reorder. */
void orc_autocorrelate(double* data, int ny, int nx, int center) {
    long np = (long)ny * nx;
    cplx* c = (cplx*)malloc(sizeof(cplx) * (size_t)np);
    for (long i = 0; i < np; ++i) c[i] = data[i];
    orc_fft2((double*)c, ny, nx, -1);
    for (long i = 0; i < np; ++i) c[i] = creal(c[i]) * creal(c[i]) + cimag(c[i]) * cimag(c[i]);
    orc_fft2((double*)c, ny, nx, +1);
    for (long i = 0; i < np; ++i) data[i] = creal(c[i]) / (double)np;
    if (center) orc_reorder(data, ny, nx, 0);
    free(c);
}

/* ------------------------------------------------------------------------- */
/* Patch model.                                                              */
/* ------------------------------------------------------------------------- */

typedef struct {
    int32_t otf_size;     /* N = 2 * pupil_pixels */
    int32_t pupil_pixels; /* n */
    int32_t patch_size;   /* image size, <= N */
    int32_t n_modes;      /* M */
    int32_t n_objects;
    int32_t n_images;     /* I, all objects and channels */
    int32_t n_channels;   /* C, all objects */
    int32_t tilt_x, tilt_y;  /* mode indices of the tilts, -1 if absent */
    int32_t n_free;       /* columns of the null-space map */
    int32_t cutout_size;  /* size of the image cutouts incl. shift margins */
    int32_t pad;
} orc_geom;

typedef struct {
    int32_t n_initial_modes;   /* MODE_START */
    int32_t n_mode_increment;  /* MODE_STEP */
    int32_t max_iterations;    /* MAX_ITER */
    int32_t min_iterations;    /* MIN_ITER */
    int32_t target_iterations; /* N_DONE_ITER */
    int32_t fd_first;          /* 1: first gradient evaluations by finite differences (as the reference) */
    double ftol;               /* FTOL */
    double eps;                /* EPS */
    double brent_tol;          /* 0.1 in conjugate_gradient.cpp:231 */
} orc_cfg;

typedef struct {
    double initial_metric;
    double final_metric;
    int32_t iterations;
    int32_t status;   /* 0 ok, 1 gave up (failCount > maxFails) */
    int32_t n_f_evals;
    int32_t n_df_evals;
    int32_t fail_count;
    int32_t n_metrics;
} orc_report;

typedef struct {
    cplx* otf;   /* N*N, centred (work / current OTF) */
    cplx* pf;    /* n*n */
    cplx* tmpc;  /* N*N */
    cplx* tmpc2; /* N*N */
    cplx* tmpc3; /* N*N */
    double* tmpd;  /* max(N,cs)^2 */
    double* tmpd2; /* max(N,cs)^2 */
    double* phi;   /* n*n */
    double* vogel; /* n*n */
    cplx* work;    /* 2*N */
} img_scratch;

typedef struct {
    orc_geom g;
    int N, n, ps, M, nObj, nImg, nCh, cs, margin;
    long N2, n2;
    /* static */
    double* modes;      /* M*n2 */
    double* pupil;      /* n2 */
    double area;
    int nPupSup; int32_t* pupSup; int32_t* pupInOtf;
    int nOtfSup; int32_t* otfSup;
    int32_t* imgObj; int32_t* imgCh;
    int32_t* objImgCount;
    double* phiFixed;   /* nCh*n2 */
    double* objWeight;  /* nObj */
    double* objGradStep;/* nObj: graddiff_step * wavelength */
    double* window; double* noiseWindow;  /* ps*ps */
    double J_T_xy[2][2], J_xy_T[2][2];
    int have_jacobian;
    /* constraints (ns_entries): alpha[row] += val * beta[col] */
    int nPar, nFree; long nnz; int32_t* nsRow; int32_t* nsCol; double* nsVal;
    /* per patch */
    float* cutouts;     /* nImg * cs * cs */
    double* phiChannel; /* nImg * n2 */
    double* otfNorm;    /* nCh */
    int32_t* curShift;  /* nImg*2: (y,x) */
    double* curTiltOffset; /* nImg*2: (y,x) currentTiltOffset */
    double* statMean; double* statStd; double* statNoise; /* nImg */
    cplx* D;            /* nImg*N2 centred image FT */
    double* ftSum;      /* nObj*N2 */
    double* regGamma;   /* nObj */
    int fixed_gamma;
    double* fixedGamma;
    /* FIT_PLANE (RF_FIT_PLANE): the fitted plane of each object, float values as
     * Object::fittedPlane, nObj * ps * ps; NULL when off */
    float* plane;
    /* warm start (INIT_FILES): the initial coefficients Solver::loadInit puts in alpha_offset
     * (solver.cpp:412, 726-733), nPar; NULL for a start at zero */
    double* initAlpha;
    /* REG_ALPHA: Solver::regAlphaWeights (solver.cpp:147-156), nPar; NULL when REG_ALPHA = 0 */
    double* regW;
    /* object work */
    cplx* P; double* Q; cplx* PQ; double* PS; double* QS; /* nObj*N2 */
    double* objMetric;
    /* image state */
    cplx* OTF;          /* nImg*N2 */
    cplx* PF;           /* nImg*n2 */
    double* PHI;        /* nImg*n2 */
    /* solver vectors */
    double* alpha; double* alphaOffset; double* gradAlpha; /* nPar */
    uint8_t* enabled;
    fft_plan planN, planPS;
    img_scratch* scr;   /* per image */
    int nthreads;
    int64_t n_f, n_df;
} orc_patch;

static void* xcalloc(size_t n, size_t s) {
    void* p = calloc(n ? n : 1, s);
    if (!p) { fprintf(stderr, "oracle: out of memory\n"); abort(); }
    return p;
}

void orc_destroy(orc_patch* p);

/* pupInOtf is derived here from pupSup exactly as Pupil::generateSupport (pupil.cpp:245-262). */
orc_patch* orc_create(const orc_geom* g, const double* modes, const double* pupil,
                      int nPupSup, const int32_t* pupSup, int nOtfSup, const int32_t* otfSup,
                      const int32_t* imgObj, const int32_t* imgCh, const double* phiFixed,
                      const double* objWeight, const double* objGradStep,
                      const double* window, const double* noiseWindow,
                      long nnz, const int32_t* nsRow, const int32_t* nsCol, const double* nsVal,
                      const double* J_T_xy /* 4 or NULL */) {
    orc_patch* p = (orc_patch*)xcalloc(1, sizeof(orc_patch));
    p->g = *g;
    p->N = g->otf_size; p->n = g->pupil_pixels; p->ps = g->patch_size; p->M = g->n_modes;
    p->nObj = g->n_objects; p->nImg = g->n_images; p->nCh = g->n_channels;
    p->cs = g->cutout_size > 0 ? g->cutout_size : g->patch_size;
    p->margin = (p->cs - p->ps) / 2;
    p->N2 = (long)p->N * p->N; p->n2 = (long)p->n * p->n;
    const long N2 = p->N2, n2 = p->n2;
    p->modes = (double*)xcalloc((size_t)p->M * n2, sizeof(double));
    memcpy(p->modes, modes, sizeof(double) * (size_t)p->M * n2);
    p->pupil = (double*)xcalloc((size_t)n2, sizeof(double));
    memcpy(p->pupil, pupil, sizeof(double) * (size_t)n2);
    p->nPupSup = nPupSup;
    p->pupSup = (int32_t*)xcalloc((size_t)nPupSup, sizeof(int32_t));
    p->pupInOtf = (int32_t*)xcalloc((size_t)nPupSup, sizeof(int32_t));
    p->area = 0;
    for (int i = 0; i < nPupSup; ++i) {
        int32_t c = pupSup[i];
        p->pupSup[i] = c;
        p->pupInOtf[i] = (c / p->n) * p->N + (c % p->n) + (p->n / 2) + (p->n / 2) * p->N;
        p->area += pupil[c];
    }
    p->nOtfSup = nOtfSup;
    p->otfSup = (int32_t*)xcalloc((size_t)nOtfSup, sizeof(int32_t));
    memcpy(p->otfSup, otfSup, sizeof(int32_t) * (size_t)nOtfSup);
    p->imgObj = (int32_t*)xcalloc((size_t)p->nImg, sizeof(int32_t));
    p->imgCh = (int32_t*)xcalloc((size_t)p->nImg, sizeof(int32_t));
    memcpy(p->imgObj, imgObj, sizeof(int32_t) * (size_t)p->nImg);
    memcpy(p->imgCh, imgCh, sizeof(int32_t) * (size_t)p->nImg);
    p->objImgCount = (int32_t*)xcalloc((size_t)p->nObj, sizeof(int32_t));
    for (int i = 0; i < p->nImg; ++i) p->objImgCount[imgObj[i]]++;
    p->phiFixed = (double*)xcalloc((size_t)p->nCh * n2, sizeof(double));
    memcpy(p->phiFixed, phiFixed, sizeof(double) * (size_t)p->nCh * n2);
    p->objWeight = (double*)xcalloc((size_t)p->nObj, sizeof(double));
    memcpy(p->objWeight, objWeight, sizeof(double) * (size_t)p->nObj);
    p->objGradStep = (double*)xcalloc((size_t)p->nObj, sizeof(double));
    memcpy(p->objGradStep, objGradStep, sizeof(double) * (size_t)p->nObj);
    long ps2 = (long)p->ps * p->ps;
    p->window = (double*)xcalloc((size_t)ps2, sizeof(double));
    p->noiseWindow = (double*)xcalloc((size_t)ps2, sizeof(double));
    memcpy(p->window, window, sizeof(double) * (size_t)ps2);
    memcpy(p->noiseWindow, noiseWindow, sizeof(double) * (size_t)ps2);
    if (J_T_xy) {
        p->have_jacobian = 1;
        p->J_T_xy[0][0] = J_T_xy[0]; p->J_T_xy[0][1] = J_T_xy[1];
        p->J_T_xy[1][0] = J_T_xy[2]; p->J_T_xy[1][1] = J_T_xy[3];
        /* invert_2x2 */
        double det = p->J_T_xy[0][0] * p->J_T_xy[1][1] - p->J_T_xy[0][1] * p->J_T_xy[1][0];
        p->J_xy_T[0][0] = p->J_T_xy[1][1] / det;
        p->J_xy_T[0][1] = -p->J_T_xy[0][1] / det;
        p->J_xy_T[1][0] = -p->J_T_xy[1][0] / det;
        p->J_xy_T[1][1] = p->J_T_xy[0][0] / det;
    }
    p->nPar = p->nImg * p->M;
    p->nFree = g->n_free;
    p->nnz = nnz;
    p->nsRow = (int32_t*)xcalloc((size_t)nnz, sizeof(int32_t));
    p->nsCol = (int32_t*)xcalloc((size_t)nnz, sizeof(int32_t));
    p->nsVal = (double*)xcalloc((size_t)nnz, sizeof(double));
    memcpy(p->nsRow, nsRow, sizeof(int32_t) * (size_t)nnz);
    memcpy(p->nsCol, nsCol, sizeof(int32_t) * (size_t)nnz);
    memcpy(p->nsVal, nsVal, sizeof(double) * (size_t)nnz);

    p->cutouts = (float*)xcalloc((size_t)p->nImg * p->cs * p->cs, sizeof(float));
    p->phiChannel = (double*)xcalloc((size_t)p->nImg * n2, sizeof(double));
    p->otfNorm = (double*)xcalloc((size_t)p->nCh, sizeof(double));
    p->curShift = (int32_t*)xcalloc((size_t)p->nImg * 2, sizeof(int32_t));
    p->curTiltOffset = (double*)xcalloc((size_t)p->nImg * 2, sizeof(double));
    p->statMean = (double*)xcalloc((size_t)p->nImg, sizeof(double));
    p->statStd = (double*)xcalloc((size_t)p->nImg, sizeof(double));
    p->statNoise = (double*)xcalloc((size_t)p->nImg, sizeof(double));
    p->D = (cplx*)xcalloc((size_t)p->nImg * N2, sizeof(cplx));
    p->ftSum = (double*)xcalloc((size_t)p->nObj * N2, sizeof(double));
    p->regGamma = (double*)xcalloc((size_t)p->nObj, sizeof(double));
    p->fixedGamma = (double*)xcalloc((size_t)p->nObj, sizeof(double));
    p->P = (cplx*)xcalloc((size_t)p->nObj * N2, sizeof(cplx));
    p->Q = (double*)xcalloc((size_t)p->nObj * N2, sizeof(double));
    p->PQ = (cplx*)xcalloc((size_t)p->nObj * N2, sizeof(cplx));
    p->PS = (double*)xcalloc((size_t)p->nObj * N2, sizeof(double));
    p->QS = (double*)xcalloc((size_t)p->nObj * N2, sizeof(double));
    p->objMetric = (double*)xcalloc((size_t)p->nObj, sizeof(double));
    p->OTF = (cplx*)xcalloc((size_t)p->nImg * N2, sizeof(cplx));
    p->PF = (cplx*)xcalloc((size_t)p->nImg * n2, sizeof(cplx));
    p->PHI = (double*)xcalloc((size_t)p->nImg * n2, sizeof(double));
    p->alpha = (double*)xcalloc((size_t)p->nPar, sizeof(double));
    p->alphaOffset = (double*)xcalloc((size_t)p->nPar, sizeof(double));
    p->gradAlpha = (double*)xcalloc((size_t)p->nPar, sizeof(double));
    p->enabled = (uint8_t*)xcalloc((size_t)p->M, 1);
    plan_init(&p->planN, p->N);
    plan_init(&p->planPS, p->ps);
    long big = N2 > (long)p->cs * p->cs ? N2 : (long)p->cs * p->cs;
    p->scr = (img_scratch*)xcalloc((size_t)p->nImg, sizeof(img_scratch));
    for (int i = 0; i < p->nImg; ++i) {
        img_scratch* s = &p->scr[i];
        s->otf = (cplx*)xcalloc((size_t)N2, sizeof(cplx));
        s->pf = (cplx*)xcalloc((size_t)n2, sizeof(cplx));
        s->tmpc = (cplx*)xcalloc((size_t)big, sizeof(cplx));
        s->tmpc2 = (cplx*)xcalloc((size_t)big, sizeof(cplx));
        s->tmpc3 = (cplx*)xcalloc((size_t)big, sizeof(cplx));
        s->tmpd = (double*)xcalloc((size_t)big, sizeof(double));
        s->tmpd2 = (double*)xcalloc((size_t)big, sizeof(double));
        s->phi = (double*)xcalloc((size_t)n2, sizeof(double));
        s->vogel = (double*)xcalloc((size_t)n2, sizeof(double));
        int mx = p->N > p->cs ? p->N : p->cs;
        s->work = (cplx*)xcalloc((size_t)4 * mx, sizeof(cplx));
    }
    p->nthreads = 1;
    return p;
}

void orc_destroy(orc_patch* p) {
    if (!p) return;
    for (int i = 0; i < p->nImg; ++i) {
        img_scratch* s = &p->scr[i];
        free(s->otf); free(s->pf); free(s->tmpc); free(s->tmpc2); free(s->tmpc3);
        free(s->tmpd); free(s->tmpd2); free(s->phi); free(s->vogel); free(s->work);
    }
    free(p->scr);
    plan_free(&p->planN); plan_free(&p->planPS);
    free(p->modes); free(p->pupil); free(p->pupSup); free(p->pupInOtf); free(p->otfSup);
    free(p->imgObj); free(p->imgCh); free(p->objImgCount); free(p->phiFixed);
    free(p->objWeight); free(p->objGradStep); free(p->window); free(p->noiseWindow);
    free(p->nsRow); free(p->nsCol); free(p->nsVal);
    free(p->cutouts); free(p->phiChannel); free(p->otfNorm); free(p->curShift);
    free(p->curTiltOffset); free(p->statMean); free(p->statStd); free(p->statNoise);
    free(p->D); free(p->ftSum); free(p->regGamma); free(p->fixedGamma); free(p->plane); free(p->initAlpha); free(p->regW);
    free(p->P); free(p->Q); free(p->PQ); free(p->PS); free(p->QS); free(p->objMetric);
    free(p->OTF); free(p->PF); free(p->PHI);
    free(p->alpha); free(p->alphaOffset); free(p->gradAlpha); free(p->enabled);
    free(p);
}

void orc_set_threads(orc_patch* p, int n) { p->nthreads = n > 0 ? n : 1; }

/* ---------------- autocorrelation of an N x N complex array (in place) --------------- */
/* FourierTransform::autocorrelate(inout, center=true), fouriertransform.hpp:281-286 */
static void autocorr_inplace(orc_patch* p, cplx* a, img_scratch* s) {
    const long N2 = p->N2;
    fft2(&p->planN, &p->planN, a, -1, s->work);
    for (long i = 0; i < N2; ++i) a[i] = creal(a[i]) * creal(a[i]) + cimag(a[i]) * cimag(a[i]);
    fft2(&p->planN, &p->planN, a, +1, s->work);
    const double nrm = 1.0 / (double)N2;
    for (long i = 0; i < N2; ++i) a[i] *= nrm;
    reorder_c(a, p->N, p->N, s->tmpc3);
}

/* SubImage::calcPFOTF (subimage.cpp:586-612) for image j, phase phi */
static void calc_pf_otf(orc_patch* p, int j, double otfNorm, const double* phi, cplx* pf, cplx* otf,
                        img_scratch* s) {
    memset(pf, 0, sizeof(cplx) * (size_t)p->n2);
    memset(otf, 0, sizeof(cplx) * (size_t)p->N2);
    for (int i = 0; i < p->nPupSup; ++i) {
        int32_t a = p->pupSup[i];
        double A = p->pupil[a];
        pf[a] = A * cos(phi[a]) + I * (A * sin(phi[a]));   /* std::polar(A, phi) */
        otf[p->pupInOtf[i]] = otfNorm * pf[a];
    }
    (void)j;
    autocorr_inplace(p, otf, s);
}

/* SubImage::calcOTF(otf, phi) (subimage.cpp:567-583) */
static void calc_otf(orc_patch* p, double otfNorm, const double* phi, cplx* otf, img_scratch* s) {
    memset(otf, 0, sizeof(cplx) * (size_t)p->N2);
    for (int i = 0; i < p->nPupSup; ++i) {
        int32_t a = p->pupSup[i];
        double A = p->pupil[a] * otfNorm;
        otf[p->pupInOtf[i]] = A * cos(phi[a]) + I * (A * sin(phi[a]));
    }
    autocorr_inplace(p, otf, s);
}

/* SubImage::calcPhi / addToPhi (subimage.cpp:509-544) */
static void calc_phi(orc_patch* p, int j, const double* a, double* phi) {
    const long n2 = p->n2;
    memcpy(phi, p->phiChannel + (long)j * n2, sizeof(double) * (size_t)n2);
    for (int m = 0; m < p->M; ++m) {
        double al = a[m];
        if (m == p->g.tilt_x) al += p->curTiltOffset[2 * j + 1];
        else if (m == p->g.tilt_y) al += p->curTiltOffset[2 * j + 0];
        if (fabs(al) > 0.0) {
            const double* mp = p->modes + (long)m * n2;
            for (long i = 0; i < n2; ++i) phi[i] = phi[i] + al * mp[i];
        }
    }
}

/* Channel::initPatch otfNormalization (channel.cpp:941-952) */
static void compute_otf_norms(orc_patch* p) {
    img_scratch* s = &p->scr[0];
    double* zero = (double*)xcalloc((size_t)p->n2, sizeof(double));
    for (int c = 0; c < p->nCh; ++c) {
        calc_pf_otf(p, 0, 1.0, zero, s->pf, s->otf, s);
        double mx = 0;
        for (long i = 0; i < p->N2; ++i) { double v = cabs(s->otf[i]); if (v > mx) mx = v; }
        p->otfNorm[c] = 1.0 / sqrt(mx);
    }
    free(zero);
}

/* ---------------- image initialisation (SubImage::initialize) ---------------- */

/* FourierTransform::noise(-1,-1) for a FULLCOMPLEX, un-reordered ps x ps transform
 * (fouriertransform.cpp:448-495) */
static double ft_noise(const cplx* ft, int ny, int nx) {
    int mask = (ny > nx ? ny : nx) / 6 + 1;
    double limits = (double)ny * nx / 4.0;
    int endX = nx - mask + 1, endY = ny - mask + 1;
    double np = 0; long cnt = 0;
    for (int x = mask; x < endX; ++x) {
        double xx = (double)(x < nx - x ? x : nx - x);
        xx *= xx;
        for (int y = mask; y < endY; ++y) {
            double yy = (double)(y < ny - y ? y : ny - y);
            if (xx + yy * yy < limits) continue;
            const cplx v = ft[(long)y * nx + x];
            np += creal(v) * creal(v) + cimag(v) * cimag(v);
            cnt++;
        }
    }
    if (cnt) np = sqrt(np / ((double)cnt * ny * nx));
    return np;
}

/* mean and stddev as ArrayStats ST_VALUES|ST_RMS (arraystats.cpp:60-80) */
static void img_stats(const double* x, long n, double* mean, double* stddev) {
    double s = 0, s2 = 0;
    for (long i = 0; i < n; ++i) { s += x[i]; s2 += x[i] * x[i]; }
    double m = s / n, r = s2 / n;
    *mean = m;
    *stddev = sqrt(r - m * m);
}

/* Object::fitAvgPlane (object.cpp:553-594): the object's images (patch views at their
 * current shifts) summed in float in image order, divided by their count in float, a plane
 * z = a*dy + b*dx + c fitted over the whole grid by least squares (redux::image::fitPlane,
 * image/utils.cpp:169-233, GSL multifit there; a 3x3 solve here) and stored without its
 * constant (subtract_mean) through makePlane (image/utils.cpp:128-147) as float. */
static void fit_avg_plane(orc_patch* p, int o) {
    const int ps = p->ps, cs = p->cs;
    const long ps2 = (long)ps * ps;
    float* acc = (float*)xcalloc((size_t)ps2, sizeof(float));
    int count = 0;
    for (int j = 0; j < p->nImg; ++j) {
        if (p->imgObj[j] != o) continue;
        const int oy = p->margin + p->curShift[2 * j + 0], ox = p->margin + p->curShift[2 * j + 1];
        const float* cut = p->cutouts + (long)j * cs * cs;
        for (int y = 0; y < ps; ++y)
            for (int x = 0; x < ps; ++x) {
                volatile float t = acc[(long)y * ps + x] + cut[(long)(oy + y) * cs + ox + x];
                acc[(long)y * ps + x] = t;
            }
        count++;
    }
    /* normal equations, unknowns (a, b, c), design columns (dy, dx, 1) */
    double A[3][4] = {{0}};
    for (int y = 0; y < ps; ++y)
        for (int x = 0; x < ps; ++x) {
            volatile float zf = acc[(long)y * ps + x] / (float)count;
            const double z = zf, r[3] = {(double)(y - ps / 2), (double)(x - ps / 2), 1.0};
            for (int i = 0; i < 3; ++i) {
                for (int k = 0; k < 3; ++k) A[i][k] += r[i] * r[k];
                A[i][3] += r[i] * z;
            }
        }
    for (int c = 0; c < 3; ++c) {            /* Gaussian elimination with partial pivoting */
        int piv = c;
        for (int i = c + 1; i < 3; ++i) if (fabs(A[i][c]) > fabs(A[piv][c])) piv = i;
        for (int k = 0; k < 4; ++k) { double t = A[c][k]; A[c][k] = A[piv][k]; A[piv][k] = t; }
        for (int i = c + 1; i < 3; ++i) {
            const double f = A[i][c] / A[c][c];
            for (int k = c; k < 4; ++k) A[i][k] -= f * A[c][k];
        }
    }
    double sol[3];
    for (int i = 2; i >= 0; --i) {
        double v = A[i][3];
        for (int k = i + 1; k < 3; ++k) v -= A[i][k] * sol[k];
        sol[i] = v / A[i][i];
    }
    float* pl = p->plane + (long)o * ps2;
    for (int y = 0; y < ps; ++y)
        for (int x = 0; x < ps; ++x)
            pl[(long)y * ps + x] = (float)(sol[0] * (double)(y - ps / 2) + sol[1] * (double)(x - ps / 2));
    free(acc);
}

void orc_set_fit_plane(orc_patch* p, int on) {
    if (on && !p->plane) p->plane = (float*)xcalloc((size_t)p->nObj * p->ps * p->ps, sizeof(float));
    if (!on && p->plane) { free(p->plane); p->plane = NULL; }
}

static int adjust_shifts(orc_patch* p, int j, const double* a);   /* SubImage::adjustShifts, below */

void orc_set_reg_alpha(orc_patch* p, const double* w) {
    if (!w) { free(p->regW); p->regW = NULL; return; }
    if (!p->regW) p->regW = (double*)xcalloc((size_t)p->nPar, sizeof(double));
    memcpy(p->regW, w, sizeof(double) * (size_t)p->nPar);
}

void orc_set_initial_alpha(orc_patch* p, const double* a) {
    if (!a) { free(p->initAlpha); p->initAlpha = NULL; return; }
    if (!p->initAlpha) p->initAlpha = (double*)xcalloc((size_t)p->nPar, sizeof(double));
    memcpy(p->initAlpha, a, sizeof(double) * (size_t)p->nPar);
}

void orc_get_plane(const orc_patch* p, float* out) {
    if (p->plane) memcpy(out, p->plane, sizeof(float) * (size_t)p->nObj * p->ps * p->ps);
}

/* SubImage::initialize(o, doReset) (subimage.cpp:155-209) with getWindowedImg (106-150);
 * returns the contribution rg to reg_gamma when doReset. */
static void init_image(orc_patch* p, int j, int doReset, double* rg_out, cplx* oldFT) {
    img_scratch* s = &p->scr[j];
    const int ps = p->ps, N = p->N, cs = p->cs;
    const long ps2 = (long)ps * ps;
    double* img = s->tmpd;
    /* the view: patch-size window at (margin + shift) inside the cutout */
    const int oy = p->margin + p->curShift[2 * j + 0];
    const int ox = p->margin + p->curShift[2 * j + 1];
    const float* cut = p->cutouts + (long)j * cs * cs;
    for (int y = 0; y < ps; ++y)
        for (int x = 0; x < ps; ++x) img[(long)y * ps + x] = (double)cut[(long)(oy + y) * cs + ox + x];
    double avg, sd;
    img_stats(img, ps2, &avg, &sd);
    if (p->plane) {   /* getWindowedImg with the object's fitted plane (subimage.cpp:117-123) */
        const float* pl = p->plane + (long)p->imgObj[j] * ps2;
        for (long i = 0; i < ps2; ++i) img[i] = (img[i] - avg - pl[i]) * p->window[i] + avg;
    } else {
        for (long i = 0; i < ps2; ++i) img[i] = (img[i] - avg) * p->window[i] + avg;
    }
    double mean, stddev;
    img_stats(img, ps2, &mean, &stddev);
    p->statMean[j] = mean;
    p->statStd[j] = stddev;
    cplx* D = p->D + (long)j * p->N2;
    if (oldFT) memcpy(oldFT, D, sizeof(cplx) * (size_t)p->N2);
    if (doReset) {
        cplx* c = s->tmpc;
        for (long i = 0; i < ps2; ++i) c[i] = (img[i] - mean) * p->noiseWindow[i];
        fft2(&p->planPS, &p->planPS, c, -1, s->work);
        double noise = ft_noise(c, ps, ps);  /* noiseFudge = 1 */
        p->statNoise[j] = noise;
        *rg_out = noise / stddev;
    }
    cplx* c2 = s->tmpc2;
    if (ps != N) {
        int off = (N - ps) / 2;
        for (long i = 0; i < p->N2; ++i) c2[i] = mean;
        for (int y = 0; y < ps; ++y)
            for (int x = 0; x < ps; ++x) c2[(long)(off + y) * N + off + x] = img[(long)y * ps + x];
    } else {
        for (long i = 0; i < p->N2; ++i) c2[i] = img[i];
    }
    fft2(&p->planN, &p->planN, c2, -1, s->work);
    reorder_c(c2, N, N, s->tmpc3);   /* REORDER_FT */
    memcpy(D, c2, sizeof(cplx) * (size_t)p->N2);
}

/* Load the cutouts of one patch and initialise everything that Channel::initPatch,
 * Object::initPatch and Solver::shiftAndInit(alpha_offset, true) set up.
 * residual_alpha: per image (y, x) channel residual tilt coefficient (residualAlpha in
 * channel.cpp:906-939); the channel phase is phi_fixed - residual_alpha * Z_tilt. */
void orc_set_images(orc_patch* p, const float* cutouts, const double* residual_alpha,
                    const double* fixed_gamma /* nObj or NULL */) {
    const long n2 = p->n2;
    memcpy(p->cutouts, cutouts, sizeof(float) * (size_t)p->nImg * p->cs * p->cs);
    for (int j = 0; j < p->nImg; ++j) {
        double* pc = p->phiChannel + (long)j * n2;
        memcpy(pc, p->phiFixed + (long)p->imgCh[j] * n2, sizeof(double) * (size_t)n2);
        if (residual_alpha) {
            double ry = residual_alpha[2 * j + 0], rx = residual_alpha[2 * j + 1];
            if (p->g.tilt_x >= 0 && fabs(rx) > 0) {
                const double* mp = p->modes + (long)p->g.tilt_x * n2;
                double res = -rx;
                for (long i = 0; i < n2; ++i) pc[i] = pc[i] + res * mp[i];
            }
            if (p->g.tilt_y >= 0 && fabs(ry) > 0) {
                const double* mp = p->modes + (long)p->g.tilt_y * n2;
                double res = -ry;
                for (long i = 0; i < n2; ++i) pc[i] = pc[i] + res * mp[i];
            }
        }
        p->curShift[2 * j] = p->curShift[2 * j + 1] = 0;
        p->curTiltOffset[2 * j] = p->curTiltOffset[2 * j + 1] = 0;
    }
    /* Solver::shiftAndInit(alpha_offset, true) after loadInit: the cutout windows follow the
     * tilts of the initial coefficients (SubImage::adjustShifts) before the images are set up */
    if (p->initAlpha)
        for (int j = 0; j < p->nImg; ++j) adjust_shifts(p, j, p->initAlpha + (long)j * p->M);
    compute_otf_norms(p);
    p->fixed_gamma = fixed_gamma != NULL;
    if (fixed_gamma) memcpy(p->fixedGamma, fixed_gamma, sizeof(double) * (size_t)p->nObj);
    /* shiftAndInit(alpha_offset = 0, doReset = true): no shift, full initialisation */
    memset(p->ftSum, 0, sizeof(double) * (size_t)p->nObj * p->N2);
    memset(p->regGamma, 0, sizeof(double) * (size_t)p->nObj);
    if (p->plane)     /* ObjectData::initPatch fits the planes before the images are set up */
        for (int o = 0; o < p->nObj; ++o) fit_avg_plane(p, o);
    double* rg = (double*)xcalloc((size_t)p->nImg, sizeof(double));
#pragma omp parallel for schedule(dynamic, 1) num_threads(p->nthreads)
    for (int j = 0; j < p->nImg; ++j) init_image(p, j, 1, &rg[j], NULL);
    for (int j = 0; j < p->nImg; ++j) {
        int o = p->imgObj[j];
        p->regGamma[o] += 0.10 * rg[j] / p->objImgCount[o];   /* Object::addRegGamma */
        const cplx* D = p->D + (long)j * p->N2;
        double* fs = p->ftSum + (long)o * p->N2;
        for (long i = 0; i < p->N2; ++i) fs[i] += creal(D[i]) * creal(D[i]) + cimag(D[i]) * cimag(D[i]);
    }
    if (p->fixed_gamma) memcpy(p->regGamma, p->fixedGamma, sizeof(double) * (size_t)p->nObj);
    free(rg);
}

/* ---------------- forward: applyAlpha + metric ---------------- */

static void apply_alpha(orc_patch* p, const double* alpha) {
    if (alpha != p->alpha) memcpy(p->alpha, alpha, sizeof(double) * (size_t)p->nPar);   /* Solver::alpha */
#pragma omp parallel for schedule(dynamic, 1) num_threads(p->nthreads)
    for (int j = 0; j < p->nImg; ++j) {
        img_scratch* s = &p->scr[j];
        double* phi = p->PHI + (long)j * p->n2;
        calc_phi(p, j, alpha + (long)j * p->M, phi);
        calc_pf_otf(p, j, p->otfNorm[p->imgCh[j]], phi, p->PF + (long)j * p->n2,
                    p->OTF + (long)j * p->N2, s);
    }
}

/* Object::initPQ + addPQ over all images (Solver::metric / calcPQ) */
static void calc_pq(orc_patch* p) {
    const long N2 = p->N2;
    for (int o = 0; o < p->nObj; ++o) {
        cplx* P = p->P + (long)o * N2;
        double* Q = p->Q + (long)o * N2;
        for (long i = 0; i < N2; ++i) { P[i] = 0; Q[i] = p->regGamma[o]; }
    }
#pragma omp parallel for schedule(static) num_threads(p->nthreads)
    for (int k = 0; k < p->nOtfSup; ++k) {
        const int32_t u = p->otfSup[k];
        for (int j = 0; j < p->nImg; ++j) {
            const int o = p->imgObj[j];
            const cplx S = p->OTF[(long)j * N2 + u];
            const cplx Dv = p->D[(long)j * N2 + u];
            p->Q[(long)o * N2 + u] += creal(S) * creal(S) + cimag(S) * cimag(S);
            p->P[(long)o * N2 + u] += conj(Dv) * S;
        }
    }
}

/* Object::calcHelpers (object.cpp:531-550) */
static void calc_helpers(orc_patch* p) {
    const long N2 = p->N2;
    for (int o = 0; o < p->nObj; ++o) {
        cplx* P = p->P + (long)o * N2; double* Q = p->Q + (long)o * N2;
        cplx* PQ = p->PQ + (long)o * N2; double* PS = p->PS + (long)o * N2; double* QS = p->QS + (long)o * N2;
        memset(PQ, 0, sizeof(cplx) * (size_t)N2);
        memset(PS, 0, sizeof(double) * (size_t)N2);
        memset(QS, 0, sizeof(double) * (size_t)N2);
        for (int k = 0; k < p->nOtfSup; ++k) {
            const int32_t u = p->otfSup[k];
            PQ[u] = P[u] * Q[u];
            PS[u] = creal(P[u]) * creal(P[u]) + cimag(P[u]) * cimag(P[u]);
            QS[u] = Q[u] * Q[u];
        }
    }
}

/* Object::calcMetric (object.cpp:597-615); Solver::metric sums weight * currentMetric */
static double calc_metric(orc_patch* p) {
    const long N2 = p->N2;
    double sum = 0;
    for (int o = 0; o < p->nObj; ++o) {
        if (p->objWeight[o] == 0.0) { p->objMetric[o] = 0; continue; }
        const double* fs = p->ftSum + (long)o * N2;
        const cplx* P = p->P + (long)o * N2;
        const double* Q = p->Q + (long)o * N2;
        double m = 0;
        for (int k = 0; k < p->nOtfSup; ++k) {
            const int32_t u = p->otfSup[k];
            m += (fs[u] - (creal(P[u]) * creal(P[u]) + cimag(P[u]) * cimag(P[u])) / Q[u]);
        }
        m /= ((double)p->ps * p->ps);
        p->objMetric[o] = m;
        sum += p->objWeight[o] * m;
    }
    if (p->regW)      /* Solver::metric: + 0.5 sum alpha^2 w (solver.cpp:804-811) */
        for (int i = 0; i < p->nPar; ++i) sum += 0.5 * p->alpha[i] * p->alpha[i] * p->regW[i];
    return sum;
}

double orc_metric(orc_patch* p, const double* alpha) {
    apply_alpha(p, alpha);
    calc_pq(p);
    p->n_f++;
    return calc_metric(p);
}

/* ---------------- gradients ---------------- */

/* SubImage::calcVogelWeight (subimage.cpp:348-390), writes s->vogel */
static void calc_vogel_weight(orc_patch* p, int j, img_scratch* s) {
    const int N = p->N, n = p->n;
    const long N2 = p->N2;
    const int o = p->imgObj[j];
    const cplx* otf = p->OTF + (long)j * N2;
    const cplx* ft = p->D + (long)j * N2;
    const cplx* pf = p->PF + (long)j * p->n2;
    const cplx* pq = p->PQ + (long)o * N2;
    const double* psv = p->PS + (long)o * N2;
    const double* qs = p->QS + (long)o * N2;
    cplx* tmp = s->tmpc;   /* tmp->OTF */
    cplx* hj = s->tmpc2;
    cplx* gl = s->otf;     /* tmp->C (N2) */
    memset(tmp, 0, sizeof(cplx) * (size_t)N2);
    /* reorderInto(pf, n, n, tmp, N, N): quadrants of pf into the corners of tmp */
    {
        const int mid = n / 2;
        for (int y = 0; y < n; ++y) {
            int oy = (y < mid) ? (N - mid + y) : (y - mid);
            for (int x = 0; x < n; ++x) {
                int ox = (x < mid) ? (N - mid + x) : (x - mid);
                tmp[(long)oy * N + ox] = pf[(long)y * n + x];
            }
        }
    }
    /* hj = ift(tmp) normalised by 1/N^2 */
    memcpy(hj, tmp, sizeof(cplx) * (size_t)N2);
    fft2(&p->planN, &p->planN, hj, +1, s->work);
    for (long i = 0; i < N2; ++i) hj[i] /= (double)N2;
    memset(tmp, 0, sizeof(cplx) * (size_t)N2);
    for (int k = 0; k < p->nOtfSup; ++k) {
        const int32_t u = p->otfSup[k];
        tmp[u] = (pq[u] * ft[u] - psv[u] * otf[u]) / qs[u];
    }
    reorder_c(tmp, N, N, s->tmpc3);
    memcpy(gl, tmp, sizeof(cplx) * (size_t)N2);
    fft2(&p->planN, &p->planN, gl, +1, s->work);
    for (long i = 0; i < N2; ++i) gl[i] /= (double)N2;
    for (long i = 0; i < N2; ++i) gl[i] = hj[i] * creal(gl[i]);
    fft2(&p->planN, &p->planN, gl, -1, s->work);
    reorder_c(gl, N, N, s->tmpc3);
    for (int i = 0; i < p->nPupSup; ++i) {
        int32_t a = p->pupSup[i];
        s->vogel[a] = cimag(conj(pf[a]) * gl[p->pupInOtf[i]]) * p->pupil[a];
    }
}

/* SubImage::gradientVogel (subimage.cpp:312-326), already multiplied by weight */
static double gradient_vogel(orc_patch* p, int j, int m, img_scratch* s) {
    const int o = p->imgObj[j];
    if (p->objWeight[o] == 0) return 0;
    const double* mp = p->modes + (long)m * p->n2;
    const double scale = -2.0 * p->area / (double)p->N2;
    double ret = 0;
    for (int i = 0; i < p->nPupSup; ++i) {
        int32_t a = p->pupSup[i];
        ret += scale * s->vogel[a] * mp[a];
    }
    return ret * p->objWeight[o];
}

/* SubImage::metricChange (subimage.cpp:261-278) */
static double metric_change(orc_patch* p, int j, const cplx* newOTF) {
    const int o = p->imgObj[j];
    const long N2 = p->N2;
    const cplx* oldOTF = p->OTF + (long)j * N2;
    const cplx* P = p->P + (long)o * N2;
    const cplx* ft = p->D + (long)j * N2;
    const double* Q = p->Q + (long)o * N2;
    double dl = 0;
    for (int k = 0; k < p->nOtfSup; ++k) {
        const int32_t u = p->otfSup[k];
        cplx dsj = newOTF[u] - oldOTF[u];
        cplx dp = conj(ft[u]) * dsj;
        double dq = 2.0 * (creal(oldOTF[u]) * creal(dsj) + cimag(oldOTF[u]) * cimag(dsj)) +
                    (creal(dsj) * creal(dsj) + cimag(dsj) * cimag(dsj));
        double dn = 2.0 * (creal(dp) * creal(P[u]) + cimag(dp) * cimag(P[u])) +
                    (creal(dp) * creal(dp) + cimag(dp) * cimag(dp));
        double pn = creal(P[u]) * creal(P[u]) + cimag(P[u]) * cimag(P[u]);
        dl -= (Q[u] * dn - dq * pn) / (Q[u] * (Q[u] + dq));
    }
    return dl / (double)N2;
}

/* SubImage::gradientFiniteDifference (subimage.cpp:281-292) */
static double gradient_fd(orc_patch* p, int j, int m, img_scratch* s) {
    const int o = p->imgObj[j];
    if (p->objWeight[o] == 0) return 0;
    const double h = p->objGradStep[o];
    double* tphi = s->phi;
    memcpy(tphi, p->PHI + (long)j * p->n2, sizeof(double) * (size_t)p->n2);
    const double* mp = p->modes + (long)m * p->n2;
    for (long i = 0; i < p->n2; ++i) tphi[i] = tphi[i] + h * mp[i];
    calc_otf(p, p->otfNorm[p->imgCh[j]], tphi, s->tmpc, s);
    return metric_change(p, j, s->tmpc) / h * p->objWeight[o];
}

/* Solver::gradient (solver.cpp:860-894): per image, per enabled mode.
 * method 1 = finite differences, 2 = Vogel.  grad is in alpha space (nPar). */
static void gradient_alpha(orc_patch* p, int method, double* g) {
    /* Solver::gradient (solver.cpp:860-894): alpha * w with REG_ALPHA, zero otherwise; the
     * enabled modes' entries are then overwritten (assigned, not added) by the data term, so
     * the regularisation reaches only the modes not yet enabled */
    if (p->regW) for (int i = 0; i < p->nPar; ++i) g[i] = p->alpha[i] * p->regW[i];
    else memset(g, 0, sizeof(double) * (size_t)p->nPar);
#pragma omp parallel for schedule(dynamic, 1) num_threads(p->nthreads)
    for (int j = 0; j < p->nImg; ++j) {
        img_scratch* s = &p->scr[j];
        const int o = p->imgObj[j];
        if (method == 2) calc_vogel_weight(p, j, s);
        for (int m = 0; m < p->M; ++m) {
            if (!p->enabled[m]) continue;
            double v = (method == 2) ? gradient_vogel(p, j, m, s) : gradient_fd(p, j, m, s);
            g[(long)j * p->M + m] = p->objWeight[o] * v;
        }
    }
}

/* my_df in alpha space: applyAlpha, calcPQ (with helpers), gradient.
 * enabled: M flags (NULL = all); returns the metric at alpha as a by-product. */
double orc_gradient(orc_patch* p, const double* alpha, const uint8_t* enabled, int method,
                    double* grad) {
    for (int m = 0; m < p->M; ++m) p->enabled[m] = enabled ? enabled[m] : 1;
    apply_alpha(p, alpha);
    calc_pq(p);
    calc_helpers(p);
    gradient_alpha(p, method, grad);
    p->n_df++;
    return calc_metric(p);
}

/* ---------------- constraints ---------------- */

/* Constraints::apply: out[col] = sum val * in[row] (constraints.hpp:128-133) */
static void cons_apply(const orc_patch* p, const double* in, double* out) {
    memset(out, 0, sizeof(double) * (size_t)p->nFree);
    for (long e = 0; e < p->nnz; ++e) out[p->nsCol[e]] += p->nsVal[e] * in[p->nsRow[e]];
}

/* Constraints::reverseAndAdd: out = offset + N in (constraints.hpp:141-146) */
static void cons_reverse_add(const orc_patch* p, const double* in, const double* offset, double* out) {
    memcpy(out, offset, sizeof(double) * (size_t)p->nPar);
    for (long e = 0; e < p->nnz; ++e) out[p->nsRow[e]] += p->nsVal[e] * in[p->nsCol[e]];
}

void orc_cons_apply(const orc_patch* p, const double* in, double* out) { cons_apply(p, in, out); }
void orc_cons_reverse_add(const orc_patch* p, const double* in, const double* off, double* out) {
    cons_reverse_add(p, in, off, out);
}

/* ---------------- the solver (Solver::run with conjugate_rdx) ---------------- */

/* Callbacks of orc_cg_minimize: the same sequential solver on a caller's metric and gradient
 * (in place of a patch), e.g. to inject failures. */
typedef double (*orc_f_cb)(const double* x, void* user);
typedef void (*orc_df_cb)(const double* x, int32_t method, int32_t mode_count, double* g, void* user);
typedef void (*orc_shift_cb)(const double* x, void* user);

typedef struct {
    orc_patch* p;     /* NULL when the callbacks below drive the solver */
    int gradMethod;   /* 1 FD, 2 Vogel */
    double* beta_tmp;
    double* metrics; int nMetrics; int capMetrics;
    int logEvals; double* evalLog; int nEval; int capEval; /* (kind, step, f) */
    orc_f_cb cb_f; orc_df_cb cb_df; orc_shift_cb cb_shift; void* user;
    int modeCount;    /* enabled modes of the current stage (passed to cb_df) */
    int64_t cb_nf, cb_ndf;
} solver_ctx;

/* my_f: applyBeta + metric */
static double my_f(solver_ctx* c, const double* b) {
    if (c->cb_f) {
        c->cb_nf++;
        return c->cb_f(b, c->user);
    }
    orc_patch* p = c->p;
    cons_reverse_add(p, b, p->alphaOffset, p->alpha);
    double f = orc_metric(p, p->alpha);
    return f;
}

/* my_df: applyBeta + calcPQ + gradient; grad in beta space */
static void my_df(solver_ctx* c, const double* b, double* df) {
    if (c->cb_df) {
        c->cb_ndf++;
        c->cb_df(b, c->gradMethod, c->modeCount, df, c->user);
        return;
    }
    orc_patch* p = c->p;
    cons_reverse_add(p, b, p->alphaOffset, p->alpha);
    apply_alpha(p, p->alpha);
    calc_pq(p);
    calc_helpers(p);
    gradient_alpha(p, c->gradMethod, p->gradAlpha);
    cons_apply(p, p->gradAlpha, df);
    p->n_df++;
}

/* my_fdf: applyBeta, metric, gradient with the helpers left from the last calcPQ
 * (solver.cpp:237-243).  The gradient it leaves is overwritten by the first statement
 * of conjugate_rdx_iterate before anything reads it, so only f is needed here. */
static double my_fdf(solver_ctx* c, const double* b, double* df) {
    double f = my_f(c, b);
    (void)df;
    return f;
}

typedef struct {
    int n;
    int iter;
    double step, tol, pnorm, g0norm;
    double *x1, *p, *g0, *dx;
} cg_state;

/* value_at (conjugate_gradient.cpp:115-118): f(x - step*lambda*p) */
static double value_at(solver_ctx* c, cg_state* st, const double* x, double step, double lambda) {
    for (int i = 0; i < st->n; ++i) {
        st->dx[i] = 0.0 + (-step * lambda) * st->p[i];   /* take_step */
        st->x1[i] = x[i] + 1.0 * st->dx[i];
    }
    double f = my_f(c, st->x1);
    if (c->logEvals) {
        if (c->nEval + 1 > c->capEval) {
            c->capEval = c->capEval ? 2 * c->capEval : 1024;
            c->evalLog = (double*)realloc(c->evalLog, sizeof(double) * 2 * (size_t)c->capEval);
        }
        c->evalLog[2 * c->nEval] = step;
        c->evalLog[2 * c->nEval + 1] = f;
        c->nEval++;
    }
    return f;
}

#define SIGNX(a, b) ((b) >= 0.0 ? fabs(a) : -fabs(a))
#define TINY 1.0E-32
static const double GOLD = 1.6180339887498949025257;  /* (1+sqrt(5))/2 */

/* redux::math::bracket (helpers.cpp:58-129), limit = 100 */
static void bracket(solver_ctx* c, cg_state* st, const double* x, double lambda, double* a, double* b,
                    double* mid, double* fa, double* fb, double* fmid) {
    const int limit = 100;
    double u, fu, ulim;
    if (*fb > *fa) {
        double t = *a; *a = *b; *b = t;
        t = *fa; *fa = *fb; *fb = t;
    }
    *mid = *b + GOLD * (*b - *a);
    *fmid = value_at(c, st, x, *mid, lambda);
    while (*fb > *fmid) {
        double r = (*b - *a) * (*fb - *fmid);
        double q = (*b - *mid) * (*fb - *fa);
        double mx = fabs(q - r) > TINY ? fabs(q - r) : TINY;
        u = (*b) - ((*b - *mid) * q - (*b - *a) * r) / (2.0 * SIGNX(mx, q - r));
        ulim = *b + limit * (*mid - *b);
        if ((*b - u) * (u - *mid) > 0.0) {
            fu = value_at(c, st, x, u, lambda);
            if (fu < *fmid) {
                *a = *b; *b = u; *fa = *fb; *fb = fu;
                break;
            } else if (fu > *fb) {
                *mid = u; *fmid = fu;
                break;
            }
            u = *mid + GOLD * (*mid - *b);
            fu = value_at(c, st, x, u, lambda);
        } else if ((*mid - u) * (u - ulim) > 0.0) {
            fu = value_at(c, st, x, u, lambda);
            if (fu < *fmid) {
                /* SHFT(b, mid, u, mid + GOLD*(mid-b)); SHFT(fb, fmid, fu, f(u)) */
                *b = *mid; *mid = u; u = *mid + GOLD * (*mid - *b);
                *fb = *fmid; *fmid = fu; fu = value_at(c, st, x, u, lambda);
            }
        } else if ((*mid - ulim) * (ulim - u) >= 0.0) {
            u = ulim;
            fu = value_at(c, st, x, u, lambda);
        } else {
            u = *mid + GOLD * (*mid - *b);
            fu = value_at(c, st, x, u, lambda);
        }
        *a = *b; *b = *mid; *mid = u;
        *fa = *fb; *fb = *fmid; *fmid = fu;
    }
    if (*a > *b) { double t = *a; *a = *b; *b = t; t = *fa; *fa = *fb; *fb = t; }
    if (*mid > *b) { double t = *mid; *mid = *b; *b = t; t = *fmid; *fmid = *fb; *fb = t; }
    if (*mid < *a) { double t = *mid; *mid = *a; *a = t; t = *fmid; *fmid = *fa; *fa = t; }
}

/* redux::math::brent (helpers.cpp:133-215), limit = 100 */
static void brent(solver_ctx* c, cg_state* st, const double* xv, double lambda, double ax, double bx,
                  double* x, double* fx, double tol) {
    const int limit = 100;
    const double CGOLD = 2.0 - GOLD;
    double a = ax < bx ? ax : bx;
    double b = ax > bx ? ax : bx;
    double u, v, w;
    u = v = w = *x;
    double fu, fv, fw;
    fu = fv = fw = *fx = value_at(c, st, xv, *x, lambda);
    double d = 0.0, e = 0.0;
    for (int iter = 1; iter <= limit; ++iter) {
        double xm = 0.5 * (a + b);
        double tol1 = tol * fabs(*x) + TINY;
        double tol2 = 2.0 * tol1;
        if (fabs(*x - xm) <= (tol2 - 0.5 * (b - a))) return;
        if (fabs(e) > tol1) {
            double r = (*x - w) * (*fx - fv);
            double q = (*x - v) * (*fx - fw);
            double pp = (*x - v) * q - (*x - w) * r;
            q = 2.0 * (q - r);
            if (q > 0.0) pp = -pp;
            q = fabs(q);
            double etemp = e;
            e = d;
            if (fabs(pp) >= fabs(0.5 * q * etemp) || pp <= q * (a - *x) || pp >= q * (b - *x)) {
                e = (*x >= xm ? a - *x : b - *x);
                d = CGOLD * e;
            } else {
                d = pp / q;
                u = *x + d;
                if (u - a < tol2 || b - u < tol2) d = SIGNX(tol1, xm - *x);
            }
        } else {
            e = (*x >= xm ? a - *x : b - *x);
            d = CGOLD * e;
        }
        if (fabs(d) < tol1) d *= (tol1 / fabs(d));
        u = ((fabs(d) >= tol1) ? *x + d : *x + SIGNX(tol1, d));
        fu = value_at(c, st, xv, u, lambda);
        if (fu <= *fx) {
            if (u >= *x) a = *x; else b = *x;
            v = w; w = *x; *x = u;
            fv = fw; fw = *fx; *fx = fu;
        } else {
            if (u < *x) a = u; else b = u;
            if (fu <= fw || w == *x) {
                v = w; w = u; fv = fw; fw = fu;
            } else if (fu <= fv || v == *x || v == w) {
                v = u; fv = fu;
            }
        }
    }
    fprintf(stderr, "Error in brent: too many iterations!\n");
}

#define RDX_SUCCESS 0
#define RDX_ENOPROG 27
#define RDX_FAILURE (-1)

/* gsl_blas_dnrm2: the scaled sum of squares of the reference BLAS dnrm2 */
static double dnrm2(const double* v, int n) {
    double scale = 0.0, ssq = 1.0;
    if (n == 1) return fabs(v[0]);
    for (int i = 0; i < n; ++i) {
        if (v[i] != 0.0) {
            double ax = fabs(v[i]);
            if (scale < ax) { ssq = 1.0 + ssq * (scale / ax) * (scale / ax); scale = ax; }
            else ssq += (ax / scale) * (ax / scale);
        }
    }
    return scale * sqrt(ssq);
}

/* conjugate_rdx_iterate (conjugate_gradient.cpp:128-256) */
static int cg_iterate(solver_ctx* c, cg_state* st, double* x, double* f, double* gradient, double* dx) {
    const int n = st->n;
    my_df(c, x, gradient);
    double pnorm = st->pnorm;
    double g0norm = st->g0norm;
    double g1norm = dnrm2(gradient, n);
    double pg;
    if (st->iter++ == 0) {
        memcpy(st->p, gradient, sizeof(double) * (size_t)n);
        pnorm = st->pnorm = g1norm;
        pg = g1norm * g1norm;
    } else {
        if (g0norm == 0.0) {
            memset(dx, 0, sizeof(double) * (size_t)n);
            return RDX_ENOPROG;
        }
        double g0g1 = 0;
        for (int i = 0; i < n; ++i) {
            double tmp = st->g0[i] - gradient[i];
            g0g1 += tmp * gradient[i];
            st->g0[i] = tmp;
        }
        double beta = g0g1 / (g0norm * g0norm);
        for (int i = 0; i < n; ++i) st->p[i] = gradient[i] - beta * st->p[i];
        pnorm = st->pnorm = dnrm2(st->p, n);
        pg = 0;
        for (int i = 0; i < n; ++i) pg += st->p[i] * gradient[i];
    }
    double lambda = (pg >= 0.0) ? +1.0 / pnorm : -1.0 / pnorm;
    if (pnorm == 0.0) {
        memset(dx, 0, sizeof(double) * (size_t)n);
        return RDX_ENOPROG;
    }
    double fa = *f, fb, fc;
    double stepa = 0.0, stepb, stepc = 1E-21 / lambda;
    fc = value_at(c, st, x, stepc, lambda);
    bracket(c, st, x, lambda, &stepa, &stepc, &stepb, &fa, &fc, &fb);
    brent(c, st, x, lambda, stepa, stepc, &stepb, &fb, c->p ? 0.1 : 0.1);
    for (int i = 0; i < n; ++i) {
        dx[i] = 0.0 + (-stepb * lambda) * st->p[i];
        st->x1[i] = x[i] + 1.0 * dx[i];
    }
    memcpy(x, st->x1, sizeof(double) * (size_t)n);
    *f = fb;
    st->step = 0.5 * (fabs(stepb) > 2.0E-9 ? fabs(stepb) : 2.0E-9);
    st->g0norm = g1norm;
    memcpy(st->g0, gradient, sizeof(double) * (size_t)n);
    st->iter = st->iter % n;
    return RDX_SUCCESS;
}

static void push_metric(solver_ctx* c, double v) {
    if (c->nMetrics + 1 > c->capMetrics) {
        c->capMetrics = c->capMetrics ? 2 * c->capMetrics : 256;
        c->metrics = (double*)realloc(c->metrics, sizeof(double) * (size_t)c->capMetrics);
    }
    c->metrics[c->nMetrics++] = v;
}

/* SubImage::adjustShifts (subimage.cpp:444-480); returns 1 if the image was shifted */
static int adjust_shifts(orc_patch* p, int j, const double* a) {
    if (!p->have_jacobian || p->g.tilt_x < 0 || p->g.tilt_y < 0) return 0;
    const double ay = a[p->g.tilt_y] + p->curTiltOffset[2 * j + 0];
    const double ax = a[p->g.tilt_x] + p->curTiltOffset[2 * j + 1];
    /* alphaToShift: (y, x) = (ax J[1][0] + ay J[1][1], ax J[0][0] + ay J[0][1]) */
    double sy = ax * p->J_T_xy[1][0] + ay * p->J_T_xy[1][1];
    double sx = ax * p->J_T_xy[0][0] + ay * p->J_T_xy[0][1];
    int ty = -(int)lround(sy), tx = -(int)lround(sx);
    int act[2] = {0, 0};
    int want[2] = {ty, tx};
    for (int d = 0; d < 2; ++d) {
        int nsh = want[d];
        if (!nsh) continue;
        int first = p->margin + p->curShift[2 * j + d];
        int last = first + p->ps - 1;
        if (nsh + first < 0) nsh = -first;
        if (abs(nsh + last) >= p->cs) nsh = p->cs - last - 1;
        act[d] = nsh;
    }
    if (act[0] || act[1]) {
        p->curShift[2 * j + 0] += act[0];
        p->curShift[2 * j + 1] += act[1];
        /* shiftToAlpha */
        double dy = act[1] * p->J_xy_T[1][0] + act[0] * p->J_xy_T[1][1];
        double dxv = act[1] * p->J_xy_T[0][0] + act[0] * p->J_xy_T[0][1];
        p->curTiltOffset[2 * j + 0] += dy;
        p->curTiltOffset[2 * j + 1] += dxv;
        return 1;
    }
    return 0;
}

/* Solver::shiftAndInit(a, false) + Object::reInitialize (object.cpp:885-904) */
static void shift_and_init(orc_patch* p, const double* a) {
    int* shifted = (int*)xcalloc((size_t)p->nObj, sizeof(int));
    for (int j = 0; j < p->nImg; ++j)
        if (adjust_shifts(p, j, a + (long)j * p->M)) shifted[p->imgObj[j]] = 1;
    for (int o = 0; o < p->nObj; ++o) {
        if (!shifted[o]) continue;
        if (p->plane) fit_avg_plane(p, o);   /* Object::reInitialize refits the plane */
        for (int j = 0; j < p->nImg; ++j) {
            if (p->imgObj[j] != o) continue;
            cplx* oldFT = p->scr[j].tmpc3;   /* reused after init_image's reorder */
            cplx* keep = (cplx*)xcalloc((size_t)p->N2, sizeof(cplx));
            init_image(p, j, 0, NULL, keep);
            (void)oldFT;
            const cplx* D = p->D + (long)j * p->N2;
            double* fs = p->ftSum + (long)o * p->N2;
            for (long i = 0; i < p->N2; ++i)      /* Object::addDiffToFT */
                fs[i] += (creal(D[i]) * creal(D[i]) + cimag(D[i]) * cimag(D[i])) -
                         (creal(keep[i]) * creal(keep[i]) + cimag(keep[i]) * cimag(keep[i]));
            free(keep);
        }
    }
    free(shifted);
}

/* The stage loop of Solver::run (solver.cpp:330-580) with GETSTEP = conjugate_gradient, on
 * beta (n free parameters) of M modes.  With a patch it evaluates the patch (applyBeta, metric,
 * gradient; shiftAndInit between stages); with callbacks it calls them.  Leaves the final
 * point in x_out and returns the GSL status of the last iteration. */
static int run_stages(solver_ctx* c, const orc_cfg* cfg, int nFree, int M, double gradScale, double* x_out,
                      orc_report* rep) {
    orc_patch* p = c->p;
    cg_state st;
    memset(&st, 0, sizeof(st));
    st.n = nFree;
    st.x1 = (double*)xcalloc((size_t)nFree, sizeof(double));
    st.p = (double*)xcalloc((size_t)nFree, sizeof(double));
    st.g0 = (double*)xcalloc((size_t)nFree, sizeof(double));
    st.dx = (double*)xcalloc((size_t)nFree, sizeof(double));
    double* x = (double*)xcalloc((size_t)nFree, sizeof(double));
    double* gradient = (double*)xcalloc((size_t)nFree, sizeof(double));
    double* dx = (double*)xcalloc((size_t)nFree, sizeof(double));
    double* beta_init = (double*)xcalloc((size_t)nFree, sizeof(double));
    if (p) memset(p->enabled, 0, (size_t)M);
    c->modeCount = 0;
    double sf = 0;
    double previousMetric = 0, thisMetric = 0, gradNorm = 0;
    double tol = 1.0E-1;
    int failCount = 0, totalIterations = 0, maxIterations = 10, maxFails = 3;
    int status = 0;
    /* loadInit: alpha_offset = the initial coefficients (zero without them);
     * shiftAndInit(alpha_offset, true) was done by orc_set_images. */
    double initialMetric = my_f(c, beta_init);
    push_metric(c, initialMetric);
    int exitLoop = 0;
    for (int modeCount = cfg->n_initial_modes; !exitLoop; modeCount += cfg->n_mode_increment) {
        if (modeCount > M) modeCount = M;
        if (p)
            for (int m = 0; m < modeCount; ++m) p->enabled[m] = 1;
        c->modeCount = modeCount;
        if (modeCount == M || cfg->max_iterations == 0) {
            exitLoop = 1;
            tol = cfg->ftol;
            maxIterations = cfg->max_iterations;
        }
        /* gsl_multimin_fdfminimizer_set -> conjugate_rdx_set */
        memcpy(x, beta_init, sizeof(double) * (size_t)nFree);
        memset(dx, 0, sizeof(double) * (size_t)nFree);
        st.iter = 0;
        sf = my_fdf(c, x, gradient);
        int iter = 0, successCount = 0, done = 0;
        while ((!done || iter < cfg->min_iterations) && iter < maxIterations) {
            iter++;
            status = cg_iterate(c, &st, x, &sf, gradient, dx);
            if (failCount > maxFails) {
                status = RDX_FAILURE;
                exitLoop = 1;
                done = 1;
                break;
            }
            c->gradMethod = 2;   /* switch to Vogel after the first iteration */
            if (status == RDX_ENOPROG) { failCount++; break; }
            thisMetric = sf;
            if (!isfinite(thisMetric)) { failCount++; break; }
            push_metric(c, thisMetric);
            gradNorm = dnrm2(gradient, nFree) * gradScale;
            if (!isfinite(gradNorm)) { failCount++; break; }
            if (gradNorm < cfg->ftol) { exitLoop = 1; done = 1; break; }
            if (iter > 1) {
                double rc = 2.0 * fabs(thisMetric - previousMetric) /
                            (fabs(thisMetric) + fabs(previousMetric) + cfg->eps);
                if (rc < tol) {
                    if (++successCount >= cfg->target_iterations) { successCount = 0; done = 1; }
                } else {
                    successCount = 0;
                }
            }
            previousMetric = thisMetric;
        }
        thisMetric = my_f(c, x);
        totalIterations += iter;
        if (!exitLoop) {
            if (p) {
                shift_and_init(p, p->alpha);
                memcpy(p->alphaOffset, p->alpha, sizeof(double) * (size_t)p->nPar);
            } else if (c->cb_shift) {
                c->cb_shift(x, c->user);
            }
        }
    }
    memcpy(x_out, x, sizeof(double) * (size_t)nFree);
    if (rep) {
        rep->initial_metric = initialMetric;
        rep->final_metric = thisMetric;
        rep->iterations = totalIterations;
        rep->status = (status == RDX_FAILURE) ? 1 : 0;
        rep->n_f_evals = (int32_t)(p ? p->n_f : c->cb_nf);
        rep->n_df_evals = (int32_t)(p ? p->n_df : c->cb_ndf);
        rep->fail_count = failCount;
        rep->n_metrics = c->nMetrics;
    }
    free(st.x1); free(st.p); free(st.g0); free(st.dx);
    free(x); free(gradient); free(dx); free(beta_init);
    return status;
}

static void copy_logs(solver_ctx* c, double* metrics_out, int cap_metrics, double* eval_log, int cap_eval) {
    if (metrics_out) {
        int nm = c->nMetrics < cap_metrics ? c->nMetrics : cap_metrics;
        memcpy(metrics_out, c->metrics, sizeof(double) * (size_t)nm);
    }
    if (eval_log) {
        int ne = c->nEval < cap_eval ? c->nEval : cap_eval;
        memcpy(eval_log, c->evalLog, sizeof(double) * 2 * (size_t)ne);
    }
    free(c->metrics); free(c->evalLog);
}

/* Solver::run (solver.cpp:330-580) with GETSTEP = conjugate_gradient.
 * alpha_out: nPar; metrics_out: optional buffer of cap_metrics entries;
 * eval_log: optional (step, f) pairs of every line-search evaluation. */
int orc_solve(orc_patch* p, const orc_cfg* cfg, double* alpha_out, orc_report* rep,
              double* metrics_out, int cap_metrics, double* eval_log, int cap_eval) {
    const int nFree = p->nFree, nPar = p->nPar;
    solver_ctx c;
    memset(&c, 0, sizeof(c));
    c.p = p;
    c.gradMethod = cfg->fd_first ? 1 : 2;
    c.logEvals = eval_log != NULL;
    p->n_f = p->n_df = 0;
    memset(p->alpha, 0, sizeof(double) * (size_t)nPar);
    memset(p->gradAlpha, 0, sizeof(double) * (size_t)nPar);
    if (p->initAlpha) memcpy(p->alphaOffset, p->initAlpha, sizeof(double) * (size_t)nPar);
    else memset(p->alphaOffset, 0, sizeof(double) * (size_t)nPar);
    const double nTotalPixels = (double)p->nImg * p->ps * p->ps;
    double* x = (double*)xcalloc((size_t)nFree, sizeof(double));
    const int status = run_stages(&c, cfg, nFree, p->M, 1.0 / (nTotalPixels * nTotalPixels), x, rep);
    free(x);
    /* the last evaluation (at the final point) left alpha = alpha_offset + N x */
    memcpy(alpha_out, p->alpha, sizeof(double) * (size_t)nPar);
    copy_logs(&c, metrics_out, cap_metrics, eval_log, cap_eval);
    return status == RDX_FAILURE ? 1 : 0;
}

/* The same sequential solver on caller callbacks: f(x) the metric at beta = x, df(x, method,
 * mode_count, g) the gradient in beta space (method 1 finite differences, 2 Vogel; the first
 * mode_count modes enabled), shift(x) the re-shift between mode stages (may be NULL).  Writes
 * the final x (n_free), the report and the metric history. */
int orc_cg_minimize(int n_free, int n_modes, const orc_cfg* cfg, double grad_scale, orc_f_cb f, orc_df_cb df,
                    orc_shift_cb shift, void* user, double* x_out, orc_report* rep, double* metrics_out,
                    int cap_metrics) {
    if (n_free < 1 || n_modes < 1 || !cfg || !f || !df || !x_out) return -2;
    solver_ctx c;
    memset(&c, 0, sizeof(c));
    c.gradMethod = cfg->fd_first ? 1 : 2;
    c.cb_f = f; c.cb_df = df; c.cb_shift = shift; c.user = user;
    const int status = run_stages(&c, cfg, n_free, n_modes, grad_scale, x_out, rep);
    copy_logs(&c, metrics_out, cap_metrics, NULL, 0);
    return status == RDX_FAILURE ? 1 : 0;
}

/* ---------------- accessors for tests ---------------- */

void orc_get_D(const orc_patch* p, double* out) {
    memcpy(out, p->D, sizeof(cplx) * (size_t)p->nImg * p->N2);
}
void orc_get_otf(const orc_patch* p, double* out) {
    memcpy(out, p->OTF, sizeof(cplx) * (size_t)p->nImg * p->N2);
}
void orc_get_pf(const orc_patch* p, double* out) {
    memcpy(out, p->PF, sizeof(cplx) * (size_t)p->nImg * p->n2);
}
void orc_get_pq(const orc_patch* p, double* P, double* Q) {
    memcpy(P, p->P, sizeof(cplx) * (size_t)p->nObj * p->N2);
    memcpy(Q, p->Q, sizeof(double) * (size_t)p->nObj * p->N2);
}
void orc_get_ftsum(const orc_patch* p, double* out) {
    memcpy(out, p->ftSum, sizeof(double) * (size_t)p->nObj * p->N2);
}
void orc_get_gamma(const orc_patch* p, double* out) {
    memcpy(out, p->regGamma, sizeof(double) * (size_t)p->nObj);
}
void orc_get_otfnorm(const orc_patch* p, double* out) {
    memcpy(out, p->otfNorm, sizeof(double) * (size_t)p->nCh);
}
void orc_get_stats(const orc_patch* p, double* mean, double* stddev, double* noise) {
    memcpy(mean, p->statMean, sizeof(double) * (size_t)p->nImg);
    memcpy(stddev, p->statStd, sizeof(double) * (size_t)p->nImg);
    memcpy(noise, p->statNoise, sizeof(double) * (size_t)p->nImg);
}
void orc_get_shifts(const orc_patch* p, int32_t* shift, double* tiltoff) {
    memcpy(shift, p->curShift, sizeof(int32_t) * 2 * (size_t)p->nImg);
    memcpy(tiltoff, p->curTiltOffset, sizeof(double) * 2 * (size_t)p->nImg);
}

/* Solver::shiftAndInit(alpha, false) for an external driver */
void orc_shift(orc_patch* p, const double* alpha) { shift_and_init(p, alpha); }

/* FourierTransform::reorderInto (fouriertransform.hpp:112-171) for real data: the four
 * quadrants of in (inY x inX) into the corners (center=0) or around the centre (center=1)
 * of out (outY x outX), which the caller has zeroed. */
int orc_reorder_into(const double* in, int inY, int inX, double* out, int outY, int outX, int center) {
    if (!in || !out) return 1;
    if (outY == 0 && outX == 0) { outY = inY; outX = inX; }
    if (inY > outY || inX > outX) return 2;
    if (inY == outY && inX == outX) center = 0;
    const int inMidY = inY / 2, inMidX = inX / 2, oddY = inY % 2, oddX = inX % 2;
    const int diffY = outY - inY, diffX = outX - inX, diffYh = diffY / 2, diffXh = diffX / 2;
    const int wDx = center ? diffXh : 0, eDx = center ? (diffXh - diffX) : 0;
    const int sDy = center ? diffYh * outX : 0, nDy = center ? (diffYh - diffY) * outX : 0;
    const double* southEastIn = in + inMidX + oddX;
    const double* northWestIn = in + (long)(inMidY + oddY) * inX;
    const double* northEastIn = southEastIn + (long)(inMidY + oddY) * inX;
    double* southWestOut = out + sDy + wDx;
    double* southEastOut = out + outX - inMidX - oddX + sDy + eDx;
    double* northWestOut = out + (long)(outY - inMidY - oddY) * outX + nDy + wDx;
    double* northEastOut = out + (long)(outY - inMidY - oddY + 1) * outX - inMidX - oddX + nDy + eDx;
    for (int y = 0; y < inMidY; ++y) {
        memcpy(southWestOut + (long)y * outX, northEastIn + (long)y * inX, sizeof(double) * inMidX);
        memcpy(southEastOut + (long)y * outX, northWestIn + (long)y * inX, sizeof(double) * (inMidX + oddX));
    }
    for (int y = inMidY + oddY - 1; y >= 0; --y) {
        memcpy(northEastOut + (long)y * outX, in + (long)y * inX, sizeof(double) * (inMidX + oddX));
        memcpy(northWestOut + (long)y * outX, southEastIn + (long)y * inX, sizeof(double) * inMidX);
    }
    return 0;
}

/* ---------------------------------------------------------------------------------------
 * Restoration: Object::restorePatch (object.cpp:278-334) for the restored object only, with
 * SubImage::restore (subimage.cpp:242-256) and redux::image::ScharmerFilter, smooth and
 * connectedRegion (image/utils.cpp:49-57, 295-392).
 * ------------------------------------------------------------------------------------- */

/* smooth (utils.cpp:304-328): mean over [y-nY, y+nY) x [x-nX, x+nX), clipped to the array;
 * the window is asymmetric (upper bounds exclusive), as in the reference */
static void smooth_d(double* d, int ny, int nx, int nY, int nX, double* tmp) {
    for (int y = 0; y < ny; ++y) {
        const int yl = y - nY > 0 ? y - nY : 0, yh = y + nY < ny ? y + nY : ny;
        for (int x = 0; x < nx; ++x) {
            const int xl = x - nX > 0 ? x - nX : 0, xh = x + nX < nx ? x + nX : nx;
            double t = 0;
            int cnt = 0;
            for (int yy = yl; yy < yh; ++yy)
                for (int xx = xl; xx < xh; ++xx) { t += d[(long)yy * nx + xx]; cnt++; }
            tmp[(long)y * nx + x] = t / cnt;
        }
    }
    memcpy(d, tmp, sizeof(double) * (size_t)ny * nx);
}

/* connectedRegion (utils.cpp:49-57, 295-299; utils.hpp:103-108): keeps the 4-connected
 * region of points > threshold that contains the start point (which is always kept); the
 * reference recurses, here an explicit stack visits the same set */
static void connected_region(double* d, int ny, int nx, int y0, int x0, double threshold) {
    const long n = (long)ny * nx;
    uint8_t* mask = (uint8_t*)xcalloc((size_t)n, 1);
    int32_t* stack = (int32_t*)xcalloc((size_t)n * 4 + 4, sizeof(int32_t));
    long top = 0;
    stack[top++] = y0 * nx + x0;
    while (top > 0) {
        const int32_t c = stack[--top];
        const int y = c / nx, x = c % nx;
        if (mask[c]) continue;
        if (!((y == y0 && x == x0) || d[c] > threshold)) continue;
        mask[c] = 1;
        if (y + 1 < ny) stack[top++] = c + nx;
        if (y - 1 >= 0) stack[top++] = c - nx;
        if (x + 1 < nx) stack[top++] = c + 1;
        if (x - 1 >= 0) stack[top++] = c - 1;
    }
    for (long i = 0; i < n; ++i) d[i] *= mask[i];
    free(stack);
    free(mask);
}

/* ScharmerFilter (utils.cpp:334-392) on a centred N x N transform */
static void scharmer_filter(cplx* data, const double* q2, int N, double noise_power, double frequency_cutoff) {
    const long N2 = (long)N * N;
    const double hi = 1.0, lo = 0.2;
    const double noiseFactor = noise_power * N * N;
    double* pt = (double*)xcalloc((size_t)N2, sizeof(double));
    double* rr = (double*)xcalloc((size_t)N2, sizeof(double));
    double* tmp = (double*)xcalloc((size_t)N2, sizeof(double));
    for (long i = 0; i < N2; ++i) pt[i] = (creal(data[i]) * creal(data[i]) + cimag(data[i]) * cimag(data[i])) * q2[i];
    smooth_d(pt, N, N, 1, 1, tmp);
    for (long i = 0; i < N2; ++i) pt[i] = noiseFactor / pt[i];
    /* rr(y, x) = max(1 - (pt(-y, -x) + pt(y, x)) / 2, 0), indices modulo N */
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            const double m = pt[(long)((N - y) % N) * N + (N - x) % N];
            const double v = 1.0 - 0.5 * (m + pt[(long)y * N + x]);
            rr[(long)y * N + x] = v > 0.0 ? v : 0.0;
        }
    for (long i = 0; i < N2; ++i) {
        if (rr[i] < lo) rr[i] = 0.0;
        if (rr[i] > hi) rr[i] = 1.0;
    }
    rr[(long)(N / 2) * N + N / 2] = 1.0;   /* DC gain = 1 */
    connected_region(rr, N, N, N / 2, N / 2, 0.0);
    smooth_d(rr, N, N, 4, 4, tmp);
    const double fc2 = frequency_cutoff * frequency_cutoff;
    for (int y = 0; y < N; ++y)
        for (int x = 0; x < N; ++x) {
            const double r2 = (double)(y - N / 2) * (y - N / 2) + (double)(x - N / 2) * (x - N / 2);
            if (r2 > fc2) data[(long)y * N + x] = 0.0;
            else data[(long)y * N + x] *= rr[(long)y * N + x];
        }
    free(tmp);
    free(rr);
    free(pt);
}

/* Restored objects at alpha: out [nObj][ps][ps]; frequency_cutoff [nObj] (Object::
 * frequencyCutoff; the filter uses 0.9 of it); no_filter: RF_NO_FILTER */
int orc_restore(orc_patch* p, const double* alpha, const double* frequency_cutoff, int no_filter, double* out) {
    const int N = p->N;
    const long N2 = p->N2;
    apply_alpha(p, alpha);
    cplx* obj = (cplx*)xcalloc((size_t)N2, sizeof(cplx));
    double* den = (double*)xcalloc((size_t)N2, sizeof(double));
    cplx* work = (cplx*)xcalloc((size_t)2 * N, sizeof(cplx));
    for (int o = 0; o < p->nObj; ++o) {
        memset(obj, 0, sizeof(cplx) * (size_t)N2);
        memset(den, 0, sizeof(double) * (size_t)N2);
        double noiseVar = 0;
        int count = 0;
        for (int j = 0; j < p->nImg; ++j) {
            if (p->imgObj[j] != o) continue;
            const cplx* S = p->OTF + (long)j * N2;
            const cplx* Dv = p->D + (long)j * N2;
            for (int k = 0; k < p->nOtfSup; ++k) {
                const int32_t u = p->otfSup[k];
                den[u] += creal(S[u]) * creal(S[u]) + cimag(S[u]) * cimag(S[u]);
                obj[u] += conj(Dv[u]) * S[u];
            }
            noiseVar += p->statNoise[j] * p->statNoise[j];
            count++;
        }
        if (!count) continue;
        noiseVar /= count;
        for (long i = 0; i < N2; ++i) {
            obj[i] = conj(obj[i]);
            obj[i] = den[i] != 0.0 ? obj[i] / den[i] : 0.0;      /* Array::safeDivide, eps = 0 */
        }
        if (!no_filter) scharmer_filter(obj, den, N, noiseVar, 0.9 * frequency_cutoff[o]);
        /* ift: un-centre, backward transform, real part / N^2 */
        reorder_c(obj, N, N, (cplx*)p->scr[0].tmpc);
        fft2(&p->planN, &p->planN, obj, +1, work);
        const int off = (N - p->ps) / 2;
        for (int y = 0; y < p->ps; ++y)
            for (int x = 0; x < p->ps; ++x)
                out[((long)o * p->ps + y) * p->ps + x] = creal(obj[(long)(y + off) * N + x + off]) / (double)N2;
        if (p->plane) {   /* od.img += fittedPlane (object.cpp:410-413) */
            const float* pl = p->plane + (long)o * p->ps * p->ps;
            for (long i = 0; i < (long)p->ps * p->ps; ++i) out[(long)o * p->ps * p->ps + i] += pl[i];
        }
    }
    free(work);
    free(den);
    free(obj);
    return 0;
}
