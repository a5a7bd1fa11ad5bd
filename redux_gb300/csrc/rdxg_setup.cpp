// Once-per-job set-up of the static inputs: pupil sampling and geometry, the anti-aliased
// pupil and its supports, Zernike and Karhunen-Loeve mode sets with their normalisation and
// the tilt Jacobian, and the apodisation windows.  redux computes these on the master once per
// job and ships them to every worker in GlobalData; a drop-in caller may keep doing that with
// redux's own classes, or call these functions and hand the results to rdxg_create.
//
// Host code only (no CUDA calls): plain double arithmetic, no extended precision, so the
// results are the same on every host architecture.  Powers are formed by repeated
// multiplication.  The reference evaluates the Zernike radial coefficients in 100-digit
// arithmetic (include/redux/image/zernike.hpp:18); they are integers here, formed exactly in
// 128-bit integers and rounded once to double.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "../../include/rdxg.h"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kRadPerArcsec = kPi / (180.0 * 3600.0);

// Zernike::NollToNM (src/lib/image/zernike.cpp:69-80)
void noll_to_nm(int j, int* n_out, int* m_out) {
    int n = 0, len = 1;
    for (int i = 1; len < j; ++i) {
        n = i;
        len += n + 1;
    }
    const int dl = n + 1 - len + j;
    int m = 2 * ((dl + (n % 2)) / 2) + ((n % 2) ? 0 : 1) - 1;
    if (j % 2) m = -m;
    *n_out = n;
    *m_out = m;
}

// Grid::init (src/lib/image/grid.cpp:45-67) with the origin at pixel (n/2, n/2) + 0.5:
// distance and angle of pixel (y, x)
void grid_point(int n, int y, int x, double* dist, double* ang) {
    const double o = n / 2.0 + 0.5 - 0.5;
    const double dy = y - o, dx = x - o;
    if (dy == 0.0 && dx == 0.0) {
        *dist = 0.0;
        *ang = 0.0;
        return;
    }
    *dist = std::sqrt(dy * dy + dx * dx);
    *ang = std::atan2(dy, dx);
}

double ipow(double x, int k) {
    double r = 1.0;
    for (int i = 0; i < k; ++i) r *= x;
    return r;
}

unsigned __int128 binom(int n, int k) {
    if (k < 0 || k > n) return 0;
    if (k > n - k) k = n - k;
    unsigned __int128 r = 1;
    for (int i = 1; i <= k; ++i) r = r * (unsigned __int128)(n - k + i) / (unsigned __int128)i;   // exact at every step
    return r;
}

// (n-s)! / (s! ((n+m)/2-s)! ((n-m)/2-s)!) = C(n-s, s) C(n-2s, (n-m)/2-s): an integer
double radial_coefficient(int n, int am, int s) {
    const unsigned __int128 v = binom(n - s, s) * binom(n - 2 * s, (n - am) / 2 - s);
    const double d = (double)v;
    return (s % 2) ? -d : d;
}

// makePupil (src/lib/image/utils.cpp:68-124) then Pupil::normalize (pupil.cpp:280-300)
void make_pupil(int n, double radius, double inner, double* out, double* area) {
    const bool has_inner = inner > 0;
    double mn = 0, mx = 0, sum = 0;
    for (int y = 0; y < n; ++y) {
        for (int x = 0; x < n; ++x) {
            double dist, ang;
            grid_point(n, y, x, &dist, &ang);
            const double aa = std::fabs(ang);
            const double dd = (aa > kPi / 4 && aa < 3 * kPi / 4) ? std::fabs(1.0 / std::sin(aa))
                                                                 : std::fabs(1.0 / std::cos(aa));
            const double dir = dist - inner, dor = dist - radius;
            double v;
            if (has_inner && dir < -dd) v = 0.0;
            else if (dor > dd) v = 0.0;
            else if (dor < -dd && (!has_inner || dir > dd)) v = 1.0;
            else {
                double R = dor, dd2 = 2 * dd;
                if (has_inner && dor < -dd2) {
                    R = dir;
                    dd2 = -dd2;
                }
                v = 0.5 - R / dd2;
            }
            out[y * n + x] = v;
            sum += v;
            if (y == 0 && x == 0) mn = mx = v;
            mn = std::min(mn, v);
            mx = std::max(mx, v);
        }
    }
    *area = sum;
    if (mn != mx)
        for (int i = 0; i < n * n; ++i) out[i] = (out[i] - mn) / (mx - mn);
}

// Zernike mode j (Noll) before the ModeSet normalisation: Zernike::getZernike with NORMALIZE
// (zernike.cpp:234-274), scaled so that sum(Z^2 pupil) = sum(pupil)
void zernike(int j, int n, double radius, double angle, const double* pupil, double* out) {
    if (j < 2) {
        for (int i = 0; i < n * n; ++i) out[i] = (double)j;
        return;
    }
    int nn, m;
    noll_to_nm(j, &nn, &m);
    const int am = std::abs(m);
    std::vector<double> c((nn - am) / 2 + 1);
    for (int s = 0; s <= (nn - am) / 2; ++s) c[s] = radial_coefficient(nn, am, s);
    double psum = 0, zsum = 0;
    for (int y = 0; y < n; ++y) {
        for (int x = 0; x < n; ++x) {
            double dist, ang;
            grid_point(n, y, x, &dist, &ang);
            const double r = dist / radius;
            double R = 0;
            for (int s = 0; s <= (nn - am) / 2; ++s) R += c[s] * ipow(r, nn - 2 * s);
            double Z = R;
            if (m > 0) Z = R * std::cos(am * (ang - angle));
            else if (m < 0) Z = R * std::sin(am * (ang - angle));
            out[y * n + x] = Z;
            const double p = pupil[y * n + x];
            psum += p;
            zsum += Z * Z * p;
        }
    }
    const double nrm = std::sqrt(psum / zsum);
    for (int i = 0; i < n * n; ++i) out[i] *= nrm;
}

// Noll covariance of Zernike coefficients at D/r0 = 1: Zernike::calcCovariance
// (zernike.cpp:82-125)
double zernike_covariance(int i, int j) {
    if (i < 2 || j < 2) return 0.0;
    int n1, m1, n2, m2;
    noll_to_nm(i, &n1, &m1);
    noll_to_nm(j, &n2, &m2);
    if (m1 != 0 && (i + j) % 2) return 0.0;
    const int m1a = std::abs(m1), m2a = std::abs(m2);
    if (m1a != m2a) return 0.0;
    double k = std::pow(4.8 * std::exp(std::lgamma(6.0 / 5.0)), 5.0 / 6.0) *
               std::exp(std::lgamma(14.0 / 3.0) + 2.0 * std::lgamma(11.0 / 6.0)) / (std::pow(2.0, 8.0 / 3.0) * kPi);
    k *= (((n1 + n2 - 2 * m1a) / 2) % 2 ? -1.0 : 1.0) * std::sqrt((double)(n1 + 1) * (n2 + 1));
    auto sg = [](double x) { return (x <= 0 && x != std::floor(x)) ? std::copysign(1.0, std::tgamma(x)) : 1.0; };
    const double a1 = ((n1 + n2) - 5.0 / 3.0) / 2.0;
    const double a2 = ((n1 - n2) + 17.0 / 3.0) / 2.0;
    const double a3 = ((n2 - n1) + 17.0 / 3.0) / 2.0;
    const double a4 = ((n1 + n2) + 23.0 / 3.0) / 2.0;
    return k * std::exp(std::lgamma(a1) - std::lgamma(a2) - std::lgamma(a3) - std::lgamma(a4)) * sg(a1) * sg(a2) *
           sg(a3) * sg(a4);
}

// Symmetric eigen-decomposition by cyclic Jacobi rotations (A is overwritten; V holds the
// eigenvectors as columns).  Used for the covariance blocks of the KL expansion, which the
// reference decomposes with gsl_linalg_SV_decomp: for a symmetric matrix the singular values
// are |eigenvalues| and the left singular vectors the eigenvectors.
void jacobi_eigen(int n, std::vector<double>& A, std::vector<double>& V) {
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0, tot = 0;
        for (int p = 0; p < n; ++p)
            for (int q = 0; q < n; ++q) {
                const double a = A[(size_t)p * n + q];
                tot += a * a;
                if (p != q) off += a * a;
            }
        if (off <= 1e-32 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p) {
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[(size_t)p * n + q];
                if (apq == 0.0) continue;
                const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                const double theta = (aqq - app) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {   // A <- A J (columns p, q)
                    const double akp = A[(size_t)k * n + p], akq = A[(size_t)k * n + q];
                    A[(size_t)k * n + p] = c * akp - s * akq;
                    A[(size_t)k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {   // A <- J^T A (rows p, q)
                    const double apk = A[(size_t)p * n + k], aqk = A[(size_t)q * n + k];
                    A[(size_t)p * n + k] = c * apk - s * aqk;
                    A[(size_t)q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - s * vkq;
                    V[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
        }
    }
}

struct KLMode {
    double covariance = 0;
    std::vector<std::pair<int, double>> weights;   // (Noll index, coefficient)
};

// Zernike::karhunenLoeveExpansion (zernike.cpp:367-479): the reference's exchange pass makes
// the modes coupled by the covariance contiguous; each block is decomposed (values in
// decreasing order); KL mode i takes the vector whose column is i's position in its block,
// signed so that its largest coefficient is positive.
std::map<int, KLMode> kl_expansion(int first, int last) {
    std::map<int, int> mapping;
    for (int i = first; i <= last; ++i) mapping[i] = i;
    for (int i = first; i < last; ++i) {
        double cov1 = zernike_covariance(mapping[i], mapping[last]);
        for (int j = last - 1; j > i; --j) {
            const double cov2 = zernike_covariance(mapping[i], mapping[j]);
            if (cov2 == 0.0 && cov1 != 0.0) std::swap(mapping[j], mapping[j + 1]);
            else cov1 = cov2;
        }
    }
    std::map<int, int> reverse;
    for (auto& kv : mapping) reverse[kv.second] = kv.first;
    std::vector<std::pair<int, int>> blocks;
    for (int n = first; n <= last;) {
        const int b0 = n++;
        while (n <= last && zernike_covariance(mapping[n - 1], mapping[n]) != 0.0) ++n;
        blocks.emplace_back(b0, n - 1);
    }
    std::map<int, std::vector<double>> vectors;
    std::map<int, double> singular;
    for (auto& bl : blocks) {
        const int b0 = bl.first, size = bl.second - bl.first + 1;
        std::vector<double> C((size_t)size * size), V;
        for (int i = 0; i < size; ++i)
            for (int j = 0; j < size; ++j) C[(size_t)i * size + j] = zernike_covariance(mapping[b0 + i], mapping[b0 + j]);
        std::vector<double> U((size_t)size * size, 0.0);
        if (size > 1) {
            jacobi_eigen(size, C, V);
            std::vector<int> order(size);
            for (int k = 0; k < size; ++k) order[k] = k;
            std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                return std::fabs(C[(size_t)a * size + a]) > std::fabs(C[(size_t)b * size + b]);
            });
            for (int k = 0; k < size; ++k) {
                singular[b0 + k] = std::fabs(C[(size_t)order[k] * size + order[k]]);
                for (int r = 0; r < size; ++r) U[(size_t)r * size + k] = V[(size_t)r * size + order[k]];
            }
        } else {
            U[0] = 1.0;
            singular[b0] = C[0];
        }
        vectors[b0] = std::move(U);
    }
    std::map<int, KLMode> out;
    for (int i = first; i <= last; ++i) {
        const int im = reverse[i];
        const auto& bl = *std::find_if(blocks.begin(), blocks.end(),
                                       [&](const std::pair<int, int>& b) { return b.first <= im && im <= b.second; });
        const int b0 = bl.first, size = bl.second - bl.first + 1;
        const std::vector<double>& U = vectors[b0];
        const int col = im - b0;
        int big = 0;
        for (int r = 1; r < size; ++r)
            if (std::fabs(U[(size_t)r * size + col]) > std::fabs(U[(size_t)big * size + col])) big = r;
        const double sign = U[(size_t)big * size + col] < 0 ? -1.0 : 1.0;
        KLMode k;
        k.covariance = singular[im];
        for (int r = 0; r < size; ++r) k.weights.emplace_back(mapping[b0 + r], sign * U[(size_t)r * size + col]);
        out[i] = std::move(k);
    }
    return out;
}

// fitPlane (src/lib/image/utils.cpp:169-233): z = a y + b x + c over mask > 0, coordinates
// relative to (ny/2, nx/2); least squares through the 3 x 3 normal equations.  Returns the
// coefficients and chisq / samples.
void fit_plane(const double* z, const double* mask, int n, double coef[3], double* chisq) {
    double S[3][3] = {}, rhs[3] = {};
    int cnt = 0;
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
            if (!(mask[y * n + x] > 0)) continue;
            const double v[3] = {(double)(y - n / 2), (double)(x - n / 2), 1.0};
            for (int a = 0; a < 3; ++a) {
                rhs[a] += v[a] * z[y * n + x];
                for (int b = 0; b < 3; ++b) S[a][b] += v[a] * v[b];
            }
            ++cnt;
        }
    // Gaussian elimination with partial pivoting
    double M[3][4];
    for (int a = 0; a < 3; ++a) {
        for (int b = 0; b < 3; ++b) M[a][b] = S[a][b];
        M[a][3] = rhs[a];
    }
    for (int c = 0; c < 3; ++c) {
        int piv = c;
        for (int r = c + 1; r < 3; ++r)
            if (std::fabs(M[r][c]) > std::fabs(M[piv][c])) piv = r;
        for (int k = 0; k < 4; ++k) std::swap(M[c][k], M[piv][k]);
        for (int r = c + 1; r < 3; ++r) {
            const double f = M[r][c] / M[c][c];
            for (int k = c; k < 4; ++k) M[r][k] -= f * M[c][k];
        }
    }
    for (int c = 2; c >= 0; --c) {
        double v = M[c][3];
        for (int k = c + 1; k < 3; ++k) v -= M[c][k] * coef[k];
        coef[c] = v / M[c][c];
    }
    double ss = 0;
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
            if (!(mask[y * n + x] > 0)) continue;
            const double r = z[y * n + x] - (coef[0] * (y - n / 2) + coef[1] * (x - n / 2) + coef[2]);
            ss += r * r;
        }
    *chisq = cnt ? ss / cnt : 0.0;
}

// ModeSet::measureJacobian (src/lib/momfbd/modes.cpp:464-512): the two modes that fit a
// plane best are the tilts; J columns hold their x and y slopes times scale, ordered so that
// the first column is the x tilt when the two fit much better than the third.
void measure_jacobian(const double* modes, int M, const double* pupil, int n, double scale, double J[4]) {
    struct Fit { double chisq, a, b, c; int i; };
    std::vector<Fit> fits;
    for (int i = 0; i < M; ++i) {
        double coef[3], chisq;
        fit_plane(modes + (size_t)i * n * n, pupil, n, coef, &chisq);
        fits.push_back({chisq, coef[0], coef[1], coef[2], i});
    }
    std::sort(fits.begin(), fits.end(), [](const Fit& x, const Fit& y) {
        if (x.chisq != y.chisq) return x.chisq < y.chisq;
        if (x.a != y.a) return x.a < y.a;
        if (x.b != y.b) return x.b < y.b;
        if (x.c != y.c) return x.c < y.c;
        return x.i < y.i;
    });
    double Jm[2][2] = {{0, 0}, {0, 0}};
    for (int k = 0; k < 2 && k < M; ++k) {
        Jm[0][k] = scale * fits[k].b;
        Jm[1][k] = scale * fits[k].a;
    }
    if (M > 2 && 100 * fits[0].chisq < fits[2].chisq && 100 * fits[1].chisq < fits[2].chisq) {
        if (std::fabs(Jm[0][0]) / std::fabs(Jm[1][0]) < 1) {
            std::swap(Jm[0][0], Jm[0][1]);
            std::swap(Jm[1][0], Jm[1][1]);
        }
    }
    J[0] = Jm[0][0]; J[1] = Jm[0][1]; J[2] = Jm[1][0]; J[3] = Jm[1][1];
}

// centred 2-D DFT-based autocorrelation support: the OTF support is where the (linear)
// autocorrelation of the pupil embedded in an N = 2n grid exceeds the threshold
void autocorrelation(const double* pupil, int n, std::vector<double>& ac) {
    const int N = 2 * n;
    ac.assign((size_t)N * N, 0.0);
    for (int dy = -(n - 1); dy <= n - 1; ++dy)
        for (int dx = -(n - 1); dx <= n - 1; ++dx) {
            double s = 0;
            for (int y = std::max(0, dy); y < std::min(n, n + dy); ++y)
                for (int x = std::max(0, dx); x < std::min(n, n + dx); ++x)
                    s += pupil[y * n + x] * pupil[(y - dy) * n + (x - dx)];
            ac[(size_t)(dy + n) * N + (dx + n)] = s;
        }
}

}  // namespace

extern "C" {

int rdxg_pupil_size(int32_t n_pixels, double wavelength, double telescope_d, double arcsec_per_pixel,
                    double* frequency_cutoff, double* radius, int32_t* pupil_pixels) {
    static const int kGood[] = {16, 18, 20, 24, 25, 27, 30, 32, 36, 40, 45, 48, 50, 54, 60, 64, 72, 75, 80, 81,
                                90, 96, 100, 108, 120, 125, 128, 135, 144};
    if (n_pixels < 4 || !(wavelength > 0) || !(telescope_d > 0) || !(arcsec_per_pixel > 0)) return RDXG_ERR_ARG;
    const double q = wavelength / (arcsec_per_pixel * kRadPerArcsec * telescope_d);
    const double fc = (double)n_pixels / q;
    int np = n_pixels >> 2;
    const double r = fc / 2.0;
    if (np < r) {
        for (int g : kGood) {
            np = std::max(g, np);
            if (np >= r) break;
        }
    }
    if (frequency_cutoff) *frequency_cutoff = fc;
    if (radius) *radius = r;
    if (pupil_pixels) *pupil_pixels = np << 1;
    return RDXG_OK;
}

int rdxg_make_pupil(int32_t n, double radius, double inner_radius, double* pupil, double* area) {
    if (n < 1 || !(radius > 0) || inner_radius < 0 || !pupil) return RDXG_ERR_ARG;
    double a = 0;
    make_pupil(n, radius, inner_radius, pupil, &a);
    if (area) *area = a;
    return RDXG_OK;
}

int rdxg_pupil_support(const double* pupil, int32_t n, double threshold, int32_t* pupil_support,
                       int32_t* n_pupil_support, int32_t* pupil_in_otf, int32_t* otf_support, int32_t* n_otf_support,
                       double* area) {
    if (!pupil || n < 1 || !pupil_support || !n_pupil_support || !otf_support || !n_otf_support) return RDXG_ERR_ARG;
    const int N = 2 * n;
    int cnt = 0;
    double a = 0;
    for (int i = 0; i < n * n; ++i) {
        if (!(pupil[i] > threshold)) continue;
        pupil_support[cnt] = i;
        if (pupil_in_otf) pupil_in_otf[cnt] = (i / n) * N + (i % n) + (n / 2) + (n / 2) * N;
        a += pupil[i];
        ++cnt;
    }
    *n_pupil_support = cnt;
    if (area) *area = a;
    std::vector<double> ac;
    autocorrelation(pupil, n, ac);
    int k = 0;
    for (int i = 0; i < N * N; ++i)
        if (std::fabs(ac[i]) > threshold) otf_support[k++] = i;
    *n_otf_support = k;
    return RDXG_OK;
}

int rdxg_make_modes(const rdxg_mode_params* p, const int32_t* mode_list, int32_t n_modes, double* modes,
                    double* atm_rms, double* tilt_jacobian) {
    if (!p || !mode_list || n_modes < 1 || !modes) return RDXG_ERR_ARG;
    const int n = p->pupil_pixels;
    if (n < 1 || !(p->radius > 0) || !(p->wavelength > 0)) return RDXG_ERR_ARG;
    if (p->kind != RDXG_MODES_ZERNIKE && p->kind != RDXG_MODES_KL) return RDXG_ERR_ARG;
    for (int i = 0; i < n_modes; ++i)
        if (mode_list[i] < 2) return RDXG_ERR_ARG;
    const size_t n2 = (size_t)n * n;
    std::vector<double> pupil(n2);
    double area0 = 0;
    make_pupil(n, p->radius, 0.0, pupil.data(), &area0);
    double area = 0;   // the pupil-support area (Pupil::generateSupport)
    for (size_t i = 0; i < n2; ++i)
        if (pupil[i] > 1e-9) area += pupil[i];
    std::map<int, std::vector<double>> zc;
    auto z = [&](int j) -> const std::vector<double>& {
        auto it = zc.find(j);
        if (it != zc.end()) return it->second;
        std::vector<double> v(n2);
        zernike(j, n, p->radius, p->angle, pupil.data(), v.data());
        return zc.emplace(j, std::move(v)).first->second;
    };
    std::map<int, KLMode> kle;
    if (p->kind == RDXG_MODES_KL) {
        if (p->kl_first < 2 || p->kl_last < p->kl_first) return RDXG_ERR_ARG;
        for (int i = 0; i < n_modes; ++i)
            if (mode_list[i] > 3 && (mode_list[i] < p->kl_first || mode_list[i] > p->kl_last)) return RDXG_ERR_ARG;
        kle = kl_expansion(p->kl_first, p->kl_last);
    }
    std::vector<double> raw(n2);
    for (int i = 0; i < n_modes; ++i) {
        const int j = mode_list[i];
        double atm;
        if (p->kind == RDXG_MODES_ZERNIKE || j == 2 || j == 3) {
            // the tilts of a KL set stay Zernike (modes.cpp:372-376)
            raw = z(j);
            atm = std::sqrt(zernike_covariance(j, j));
        } else {
            // KL mode: the normalised Zernikes with |weight| >= cutoff, normalised over the pupil
            const KLMode& k = kle[j];
            std::fill(raw.begin(), raw.end(), 0.0);
            for (auto& w : k.weights) {
                if (std::fabs(w.second) < p->kl_cutoff) continue;
                const std::vector<double>& zz = z(w.first);
                for (size_t q = 0; q < n2; ++q) raw[q] += w.second * zz[q];
            }
            double s = 0;
            for (size_t q = 0; q < n2; ++q)
                if (pupil[q] > 0) s += raw[q] * raw[q] * pupil[q];
            const double nrm = std::sqrt(area / s);
            for (size_t q = 0; q < n2; ++q) raw[q] *= nrm;
            atm = std::sqrt(k.covariance);
        }
        // ModeSet::getNorms / normalize(1/wavelength) (modes.cpp:443-462, 524-535)
        double s = 0;
        for (size_t q = 0; q < n2; ++q)
            if (pupil[q] > 0) s += raw[q] * raw[q] * pupil[q];
        const double nrm = std::sqrt(s / area);
        double* out = modes + (size_t)i * n2;
        for (size_t q = 0; q < n2; ++q) out[q] = raw[q] * ((1.0 / p->wavelength) / nrm);
        if (atm_rms) atm_rms[i] = atm;
    }
    if (tilt_jacobian) measure_jacobian(modes, n_modes, pupil.data(), n, p->jacobian_scale, tilt_jacobian);
    return RDXG_OK;
}

int rdxg_apodization_windows(int32_t patch_size, int32_t apodization, double* window, double* noise_window) {
    if (patch_size < 1 || !window || !noise_window) return RDXG_ERR_ARG;
    // apodizeInPlace (src/lib/image/utils.cpp:584-614) on all-ones arrays, blends of
    // Solver::init (solver.cpp:113-126): patch/8 (or the APODIZATION setting) and half of it
    const int apod = apodization < 0 ? patch_size / 8 : apodization;
    auto fill = [&](double* w, int blend) {
        const int ps = patch_size;
        for (int i = 0; i < ps * ps; ++i) w[i] = 1.0;
        if (blend <= 0) return;
        const int b = std::min(blend, ps / 2);
        const int nn = b + 2;
        std::vector<double> tmp(nn, 0.0);
        const double step = kPi / (nn - 1);
        for (int i = 1; i < nn; ++i) tmp[i] = 0.5 + (-0.5) * std::cos(i * step);
        for (int r = 0; r < b; ++r)
            for (int x = 0; x < ps; ++x) {
                w[r * ps + x] *= tmp[r + 1];
                w[(ps - r - 1) * ps + x] *= tmp[r + 1];
            }
        for (int c = 0; c < b; ++c)
            for (int y = 0; y < ps; ++y) {
                w[y * ps + c] *= tmp[c + 1];
                w[y * ps + ps - c - 1] *= tmp[c + 1];
            }
    };
    fill(window, apod);
    fill(noise_window, apod / 2);
    return RDXG_OK;
}

}  // extern "C"
