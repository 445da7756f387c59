// Host-side FP64 mathematics of the regularized Brinkman kernel: closed forms,
// stable small-r expansions and the FP32 polynomial tables of the real-space
// pair kernel.  See pb_kernel_math.h.
#include "pb_kernel_math.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

namespace pb {

static const double kPi = 3.14159265358979323846264338327950288;
static const double kSqrtPi = 1.77245385090551602729816748334114518;

double phihat(double kn, double a, double d)
{
    double a1 = -std::expm1(-a * a * d * d / 4);
    return (1.0 + a1 * kn / (a * a)) * std::exp(-d * d * kn / 4);
}

// exp(2xz) erfc(z + x), zero where both are large and xz >= 0
// (cuda/periodicBrinkman.h:19-25).
static double experf(double x, double z)
{
    if ((x * z < 0) || (x * x + z * z < 700)) return std::exp(2 * x * z) * std::erfc(z + x);
    return 0.0;
}

void diffH_closed(double r, double a, double d, double* h1, double* h2)
{
    // cuda/periodicBrinkman.h:91-104
    double r2 = r * r;
    double ex = std::exp(-r2 / (d * d)) * (-std::expm1(-a * a * d * d / 4));
    double ec = std::erfc(r / d);
    double em = experf(-a * d / 2, r / d), ep = experf(a * d / 2, r / d);
    double pre = 1.0 / (8 * kPi * a * a * r2 * r);
    double g = 1.0 / (2 * a * a * d * d * d * kPi * kSqrtPi);
    double H1 = -2 * pre * ec;
    H1 -= (d * d + 2 * r2) * g / r2 * ex;
    H1 += pre * (1 + a * r + a * a * r2) * em;
    H1 += pre * (1 - a * r + a * a * r2) * ep;
    double H2 = 6 * pre / r2 * ec;
    H2 += (3 * d * d + 2 * r2) * g / (r2 * r2) * ex;
    H2 -= pre / r2 * (3 + 3 * a * r + a * a * r2) * em;
    H2 -= pre / r2 * (3 - 3 * a * r + a * a * r2) * ep;
    *h1 = H1;
    *h2 = H2;
}

void scaled_singular(double r, double a, double* rS1, double* r3S2)
{
    // r S1 = A1(u)/(4 pi), r^3 S2 = A2(u)/(4 pi), u = a r, from the singular
    // Brinkmanlet of cuda/periodicBrinkman.h:41-42; power series below u = 0.5.
    double u = a * r, A1, A2;
    if (u < 0.5) {
        double s1 = 0, s2 = 0, p = 1, fact = 2;
        for (int k = 2; k < 40; k++) {
            double sg = (k & 1) ? -1.0 : 1.0;
            double t1 = sg * (k - 1.0) * (k - 1.0) / fact * p;
            double t2 = -sg * (k - 1.0) * (k - 3.0) / fact * p;
            s1 += t1;
            s2 += t2;
            if (k > 4 && std::fabs(t1) < 1e-19 * std::fabs(s1) && std::fabs(t2) < 1e-19 * std::fabs(s2)) break;
            p *= u;
            fact *= (k + 1);
        }
        A1 = s1;
        A2 = s2;
    } else {
        double em = std::exp(-u);
        A1 = (-1 + em * (1 + u + u * u)) / (u * u);
        A2 = (3 - em * (3 + 3 * u + u * u)) / (u * u);
    }
    *rS1 = A1 / (4 * kPi);
    *r3S2 = A2 / (4 * kPi);
}

// 16-point Gauss-Legendre rule on [-1, 1].
static void gauss_legendre16(double* x, double* w)
{
    const int n = 16;
    for (int i = 0; i < n; i++) {
        double z = std::cos(kPi * (i + 0.75) / (n + 0.5)), dp = 1;
        for (int it = 0; it < 100; it++) {
            double p0 = 1, p1 = z;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (z * p1 - p0) / (z * z - 1);
            double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-17) break;
        }
        x[i] = z;
        w[i] = 2 / ((1 - z * z) * dp * dp);
    }
}

// Dimensionless moments Kt_j = int_0^inf [1 + c q^2/b^2] e^{-q^2/4} q^{2j}/(q^2+b^2) dq,
// b = a*delta, c = 1 - e^{-b^2/4}; K_j = delta^{1-2j} Kt_j.
static void scaled_moments(double b, int nj, double* Kt)
{
    double c = -std::expm1(-b * b / 4);
    if (b > 0 && b <= 3.0) {
        // Closed form: with I_j = int_0^inf e^{-q^2/4} q^{2j}/(q^2+b^2) dq,
        // I_0 = pi/(2b) e^{b^2/4} erfc(b/2) and, since q^2/(q^2+b^2) = 1 - b^2/(q^2+b^2),
        // I_j = M_{j-1} - b^2 I_{j-1} with the Gaussian moments
        // M_k = int_0^inf e^{-q^2/4} q^{2k} dq = Gamma(k + 1/2) 4^k.  Each step scales
        // the error of I_{j-1} by b^2 against a growing M, so up to b = 3 the moments
        // stay within 2e-15 of 40-digit quadrature; Kt_j = I_j + (c/b^2) I_{j+1}.
        std::vector<double> I(nj + 1);
        I[0] = kPi / (2 * b) * std::exp(b * b / 4) * std::erfc(b / 2);
        double M = kSqrtPi;  // M_0
        for (int j = 1; j <= nj; j++) {
            I[j] = M - b * b * I[j - 1];
            M *= 4.0 * (j - 0.5);  // M_j
        }
        const double cb = c / (b * b);
        for (int j = 0; j < nj; j++) Kt[j] = I[j] + cb * I[j + 1];
        return;
    }
    static double gx[16], gw[16];
    static std::once_flag once;
    std::call_once(once, [] { gauss_legendre16(gx, gw); });
    double qmax = 2 * std::sqrt((double)nj) + 18.0;
    std::vector<double> edges;
    for (double q = 0; q < qmax; q += 1.0) edges.push_back(q);
    edges.push_back(qmax);
    for (int j = -6; j <= 4; j++) {
        double e = b * std::ldexp(1.0, j);
        if (e > 0 && e < qmax) edges.push_back(e);
    }
    std::sort(edges.begin(), edges.end());
    for (int j = 0; j < nj; j++) Kt[j] = 0;
    // per interval, the 16 nodes' weighted powers advance together (independent
    // lanes), so the power chain is not one serial multiply per node and moment
    double g[16], k2[16];
    for (size_t p = 0; p + 1 < edges.size(); p++) {
        double lo = edges[p], hi = edges[p + 1];
        if (hi - lo < 1e-15) continue;
        double mid = 0.5 * (lo + hi), h = 0.5 * (hi - lo);
        for (int q = 0; q < 16; q++) {
            double k = mid + h * gx[q];
            k2[q] = k * k;
            g[q] = (1.0 + c * k2[q] / (b * b)) * std::exp(-k2[q] / 4) / (k2[q] + b * b) * gw[q] * h;
        }
        for (int j = 0; j < nj; j++) {
            double s = 0;
            for (int q = 0; q < 16; q++) {
                s += g[q];
                g[q] *= k2[q];
            }
            Kt[j] += s;
        }
    }
}

void blob_moments(double a, double delta, int nj, double* K)
{
    std::vector<double> Kt(nj);
    scaled_moments(a * delta, nj, Kt.data());
    for (int j = 0; j < nj; j++) K[j] = Kt[j] * std::pow(delta, 1.0 - 2.0 * j);
}

// Scaled series of R_delta: H1 = (1/delta) sum c1[m] rho^{2m}, H2 = (1/delta^3) sum c2[m] rho^{2m},
// rho = r/delta.  From the radial Fourier integral of the modified blob:
// H1 = 1/(2pi^2) int phihat k^2/(k^2+a^2) [j0 - j1/z](kr) dk,
// H2 = 1/(2pi^2) int phihat k^4/(k^2+a^2) [j2/z^2](kr) dk.
static void scaled_series(double b, int nterms, double* c1, double* c2)
{
    std::vector<double> Kt(nterms + 2);
    scaled_moments(b, nterms + 2, Kt.data());
    double f1 = 4.0 / 6.0;  // 4(m+1)^2/(2m+3)! at m = 0
    double f2 = 1.0 / 15.0; // 1/(2^m m! (2m+5)!!) at m = 0
    for (int m = 0; m < nterms; m++) {
        double sg = (m & 1) ? -1.0 : 1.0;
        c1[m] = sg * f1 * Kt[m + 1] / (2 * kPi * kPi);
        c2[m] = sg * f2 * Kt[m + 2] / (2 * kPi * kPi);
        f1 *= (m + 2.0) * (m + 2.0) / ((m + 1.0) * (m + 1.0) * (2 * m + 4.0) * (2 * m + 5.0));
        f2 *= 1.0 / (2.0 * (m + 1.0) * (2 * m + 7.0));
    }
}

void regularized_series(double a, double delta, int nterms, double* s1, double* s2)
{
    std::vector<double> c1(nterms), c2(nterms);
    scaled_series(a * delta, nterms, c1.data(), c2.data());
    for (int m = 0; m < nterms; m++) {
        s1[m] = c1[m] / std::pow(delta, 2.0 * m + 1);
        s2[m] = c2[m] / std::pow(delta, 2.0 * m + 3);
    }
}

void scaled_diffH(double r, double a, double delta, const double* ser1, const double* ser2, int nser,
                  double* T1, double* T2)
{
    if (r == 0) {
        *T1 = 1.0 / (8 * kPi);
        *T2 = 1.0 / (8 * kPi);
        return;
    }
    if (r < delta) {
        // S - R_delta with R_delta from its series (no 1/r^3 cancellation)
        double rs1, r3s2;
        scaled_singular(r, a, &rs1, &r3s2);
        double r2 = r * r, R1 = 0, R2 = 0, p = 1;
        for (int m = 0; m < nser; m++) {
            R1 += ser1[m] * p;
            R2 += ser2[m] * p;
            p *= r2;
        }
        *T1 = rs1 - r * R1;
        *T2 = r3s2 - r * r2 * R2;
        return;
    }
    double h1, h2;
    diffH_closed(r, a, delta, &h1, &h2);
    *T1 = r * h1;
    *T2 = r * r * r * h2;
}

namespace {

// The matrix C[j][k] = cos(pi j (2k + 1) / (2 nodes)) of the Chebyshev
// transform, as cos(pi q / (2 nodes)) at q = j (2k + 1) mod 4 nodes; built once
// per node count for the three counts the fits use, else per call.
const double* cos_matrix(int nodes, std::vector<double>& own)
{
    static std::once_flag once;
    static std::vector<double> m40, m64;
    auto fill = [](std::vector<double>& m, int n) {
        std::vector<double> ct(4 * n);
        for (int q = 0; q < 4 * n; q++) ct[q] = std::cos(kPi * q / (2.0 * n));
        m.resize((size_t)n * n);
        for (int j = 0; j < n; j++)
            for (int k = 0; k < n; k++) m[(size_t)j * n + k] = ct[(j * (2 * k + 1)) % (4 * n)];
    };
    static std::vector<double> m96;
    std::call_once(once, [&] {
        fill(m40, 40);
        fill(m64, 64);
        fill(m96, 96);
    });
    if (nodes == 40) return m40.data();
    if (nodes == 64) return m64.data();
    if (nodes == 96) return m96.data();
    fill(own, nodes);
    return own.data();
}

// Chebyshev coefficients of samples v[k] = f(node k) (c[0] halved, untruncated).
// Four coefficients are summed side by side (independent addition chains, each
// in the order k = 0, 1, ...).
std::vector<double> cheb_coeffs(const std::vector<double>& v)
{
    const int nodes = (int)v.size();
    std::vector<double> c(nodes), own;
    const double* C = cos_matrix(nodes, own);
    int j = 0;
    for (; j + 4 <= nodes; j += 4) {
        const double *r0 = C + (size_t)j * nodes, *r1 = r0 + nodes, *r2 = r1 + nodes, *r3 = r2 + nodes;
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int k = 0; k < nodes; k++) {
            s0 += v[k] * r0[k];
            s1 += v[k] * r1[k];
            s2 += v[k] * r2[k];
            s3 += v[k] * r3[k];
        }
        c[j] = s0 * 2.0 / nodes;
        c[j + 1] = s1 * 2.0 / nodes;
        c[j + 2] = s2 * 2.0 / nodes;
        c[j + 3] = s3 * 2.0 / nodes;
    }
    for (; j < nodes; j++) {
        const double* r = C + (size_t)j * nodes;
        double s = 0;
        for (int k = 0; k < nodes; k++) s += v[k] * r[k];
        c[j] = s * 2.0 / nodes;
    }
    c[0] *= 0.5;
    return c;
}

int cheb_terms(const std::vector<double>& c, double rel_tol)
{
    double cmax = 0;
    for (double v : c) cmax = std::max(cmax, std::fabs(v));
    int n = 1;
    for (int j = 0; j < (int)c.size(); j++)
        if (std::fabs(c[j]) > rel_tol * cmax) n = j + 1;
    return n;
}

std::vector<double> cheb_to_monomial(const std::vector<double>& c)
{
    const int n = (int)c.size();
    // T_{j+1} = 2 t T_j - T_{j-1}, the monomial coefficients of T_{j-1}, T_j and
    // T_{j+1} rotating through three rows
    std::vector<double> a(n, 0.0), rows(3 * (size_t)n, 0.0);
    double* T0 = rows.data();
    double* T1 = T0 + n;
    double* Tn = T1 + n;
    T0[0] = 1;
    if (n > 1) T1[1] = 1;
    for (int j = 0; j < n; j++) {
        const double* Tj = (j == 0) ? T0 : T1;
        for (int q = 0; q < n; q++) a[q] += c[j] * Tj[q];
        if (j >= 1) {
            Tn[0] = -T0[0];
            for (int q = 1; q < n; q++) Tn[q] = 2 * T1[q - 1] - T0[q];
            double* t = T0;
            T0 = T1;
            T1 = Tn;
            Tn = t;
        }
    }
    return a;
}

}  // namespace

std::vector<double> fit_chebyshev(const std::function<double(double)>& f, double lo, double hi, int nodes,
                                  double rel_tol, int max_terms)
{
    std::vector<double> v(nodes);
    for (int k = 0; k < nodes; k++) v[k] = f(lo + (hi - lo) * (std::cos(kPi * (k + 0.5) / nodes) + 1) / 2);
    std::vector<double> c = cheb_coeffs(v);
    c.resize(std::min(cheb_terms(c, rel_tol), max_terms));
    return c;
}

std::vector<double> fit_monomial(const std::function<double(double)>& f, double lo, double hi, int nodes,
                                 double rel_tol, int max_terms)
{
    return cheb_to_monomial(fit_chebyshev(f, lo, hi, nodes, rel_tol, max_terms));
}

void fit_chebyshev_pair(const std::function<void(double, double*, double*)>& f, double lo, double hi, int nodes,
                        double rel_tol, int max_terms, std::vector<double>& c1, std::vector<double>& c2)
{
    std::vector<double> v1(nodes), v2(nodes);
    for (int k = 0; k < nodes; k++) f(lo + (hi - lo) * (std::cos(kPi * (k + 0.5) / nodes) + 1) / 2, &v1[k], &v2[k]);
    c1 = cheb_coeffs(v1);
    c2 = cheb_coeffs(v2);
    const int n = std::min(std::max(cheb_terms(c1, rel_tol), cheb_terms(c2, rel_tol)), max_terms);
    c1.resize(n);
    c2.resize(n);
}

int build_tables(double a, double d, double eps, double rc, double poly_tol, PbTables* t, int max_terms,
                 bool fp64_far)
{
    if (max_terms <= 0 || max_terms > kMaxPoly) max_terms = kMaxPoly;
    if (!(a > 0) || !(d > 0) || !(rc > 0) || eps < 0) return -1;
    std::memset(t, 0, sizeof(PbTables));
    const int nser = 28;  // r/delta < 1 where the series is used: terms fall like 1/m!
    std::vector<double> sd1(nser), sd2(nser), se1(nser), se2(nser);
    regularized_series(a, d, nser, sd1.data(), sd2.data());
    auto Td = [&](double r, double* x, double* y) { scaled_diffH(r, a, d, sd1.data(), sd2.data(), nser, x, y); };
    // pieces: blob [0, rs], near [rs, r_mid], far [r_mid, rc]
    const double rs = eps > 0 ? std::min(5.6 * eps, rc) : 0.0;
    const double r_mid = std::min(rc, std::max(0.25 * rc, rs));
    const double r_far = std::min(r_mid, 0.75 * rc);   // keeps the far interval non-degenerate
    const double r_near = std::min(rs, 0.75 * r_mid);  // likewise for the near interval
    auto scale_off = [](double lo, double hi, float* scale, float* off) {
        *scale = (float)(2.0 / (hi - lo));
        *off = (float)(-(hi + lo) / (hi - lo));
    };
    {
        std::vector<double> c1, c2;
        fit_chebyshev_pair(Td, r_far, rc, 40, poly_tol, max_terms, c1, c2);
        // Terms past the 18th that are below 1e-7 of the largest coefficient
        // are dropped as well (the FP32 evaluation's own error is 1-5e-7 of
        // max |T|), so that a batch where a few instances would need 19 or 20
        // terms still runs the 18-term kernel.
        if ((int)c1.size() > kPreferredTerms) {
            double cmax = 0, tail = 0;
            for (size_t k = 0; k < c1.size(); k++) {
                const double m = std::max(std::fabs(c1[k]), std::fabs(c2[k]));
                cmax = std::max(cmax, m);
                if ((int)k >= kPreferredTerms) tail = std::max(tail, m);
            }
            if (tail <= 1e-7 * cmax) {
                c1.resize(kPreferredTerms);
                c2.resize(kPreferredTerms);
            }
        }
        std::vector<double> p1 = cheb_to_monomial(c1), p2 = cheb_to_monomial(c2);
        t->nd = (int)p1.size();
        for (int k = 0; k < t->nd; k++) {
            t->pd1[k] = (float)p1[k];
            t->pd2[k] = (float)p2[k];
        }
        scale_off(r_far, rc, &t->td_scale, &t->td_off);
    }
    auto cheb = [&](const std::function<void(double, double*, double*)>& f, double lo, double hi, float* c1,
                    float* c2, float* scale, float* off) {
        std::vector<double> q1, q2;
        fit_chebyshev_pair(f, lo, hi, 64, poly_tol, kMaxCheb, q1, q2);
        for (size_t k = 0; k < q1.size(); k++) {
            c1[k] = (float)q1[k];
            c2[k] = (float)q2[k];
        }
        scale_off(lo, hi, scale, off);
        return (int)q1.size();
    };
    t->nn = cheb(Td, r_near, r_mid, t->cn1, t->cn2, &t->tn_scale, &t->tn_off);
    if (fp64_far) {
        // the far piece again, in FP64 for the FP64 path's pairs beyond r_mid
        std::vector<double> q1, q2;
        fit_chebyshev_pair(Td, r_far, rc, 96, 1e-14, kMaxCheb64, q1, q2);
        t->nf = (int)q1.size();
        for (int k = 0; k < t->nf; k++) {
            t->cf1[k] = q1[k];
            t->cf2[k] = q2[k];
        }
        t->tf_scale = 2.0 / (rc - r_far);
        t->tf_off = -(rc + r_far) / (rc - r_far);
        t->rf2 = r_mid * r_mid;
    } else {
        t->rf2 = HUGE_VAL;  // no FP64 far series: every pair takes the closed forms
    }
    t->rc2 = (float)(rc * rc);
    t->rm2 = (float)(r_mid * r_mid);
    if (eps > 0) {
        regularized_series(a, eps, nser, se1.data(), se2.data());
        for (int m = 0; m < kNumSeries; m++) {
            t->ser1[m] = se1[m] - sd1[m];
            t->ser2[m] = se2[m] - sd2[m];
        }
        // R_eps - R_d (H1 and r^2 H2, the latter keeps the error of H2 r^2 uniform): its
        // series below eps/2, else the difference of the scaled forms (S cancels,
        // mildly, at r >= eps/2)
        auto HD = [&](double r, double* h1, double* r2h2) {
            if (r < 0.5 * eps) {
                const double r2 = r * r;
                double s1 = 0, s2 = 0, p = 1;
                for (int m = 0; m < nser; m++) {
                    s1 += (se1[m] - sd1[m]) * p;
                    s2 += (se2[m] - sd2[m]) * p;
                    p *= r2;
                }
                *h1 = s1;
                *r2h2 = r2 * s2;
                return;
            }
            double d1, d2, e1, e2;
            scaled_diffH(r, a, d, sd1.data(), sd2.data(), nser, &d1, &d2);
            scaled_diffH(r, a, eps, se1.data(), se2.data(), nser, &e1, &e2);
            *h1 = (d1 - e1) / r;
            *r2h2 = (d2 - e2) / r;
        };
        t->nb = cheb(HD, 0.0, rs, t->cb1, t->cb2, &t->tb_scale, &t->tb_off);
        t->rs2 = (float)(rs * rs);
        t->blob = 1;
        double rt = 0.8 * eps;
        t->rtiny2 = rt * rt;
        t->rtiny2f = (float)(rt * rt);
        t->self1 = t->ser1[0];
    } else {
        t->nb = 0;
        t->rs2 = 0;
        t->blob = 0;
        t->rtiny2 = 0;
        t->rtiny2f = 0;
        t->self1 = -sd1[0];  // -R_d(0): the reference's r -> 0 limit of diffH(d)
    }
    return 0;
}

}  // namespace pb
