// Host-side FP64 mathematics of the regularized Brinkman kernel.
//
// Used by the plan builder to produce, once per instance (alpha, d, eps, rc):
//   * FP32 polynomial tables of the pair kernel by pieces (far, near, blob;
//     see PbTables), so that it is evaluated with FMAs only and no piece is a
//     difference of two large terms;
//   * FP64 power series of R_eps - R_d in r^2, used below r_tiny;
//   * the self coefficient R_eps(0) - R_d(0) (or -R_d(0) for eps = 0), the
//     r -> 0 limit of cuda/periodicBrinkman.h:105-111.
//
// The pair kernel is H = diffH(r; d) - diffH(r; eps) with
// diffH(r; delta) = S(r) - R_delta(r) (cuda/periodicBrinkman.h:85-112,
// 152-176); the tensor is H1 I + H2 x x^T.
#pragma once
#include <functional>
#include <vector>

#include "pb_types.h"

namespace pb {

// Closed-form diffH of the reference (no switch radius; r > 0).
void diffH_closed(double r, double a, double d, double* h1, double* h2);
// Singular Brinkmanlet scaled: r*S1 and r^3*S2, stable for small alpha*r.
void scaled_singular(double r, double a, double* rS1, double* r3S2);
// Moments K_j = int_0^inf phihat_delta(k) k^{2j} / (k^2 + a^2) dk, j = 0..nj-1.
void blob_moments(double a, double delta, int nj, double* K);
// Series of R_delta in r^2: H1 = sum s1[m] r^{2m}, H2 = sum s2[m] r^{2m}.
void regularized_series(double a, double delta, int nterms, double* s1, double* s2);
// T1(r) = r*diffH1(r; delta), T2(r) = r^3*diffH2(r; delta), accurate for r >= 0.
// ser1/ser2: regularized_series(a, delta) (used for r < 0.25 delta).
void scaled_diffH(double r, double a, double delta, const double* ser1, const double* ser2, int nser,
                  double* T1, double* T2);
// Fourier symbol of the splitting blob (cuda/periodicBrinkman.h:189-196).
double phihat(double kn, double a, double d);

// Chebyshev fit of f on [lo, hi] at `nodes` points, truncated where the
// coefficients fall below rel_tol * max|c|; returned as monomial
// coefficients in t = (2 r - lo - hi)/(hi - lo) (lowest first).
std::vector<double> fit_monomial(const std::function<double(double)>& f, double lo, double hi, int nodes,
                                 double rel_tol, int max_terms);

// Chebyshev coefficients of f on [lo, hi] in t = (2 r - lo - hi)/(hi - lo),
// truncated as fit_monomial does; f(r) = sum_k c[k] T_k(t).
std::vector<double> fit_chebyshev(const std::function<double(double)>& f, double lo, double hi, int nodes,
                                  double rel_tol, int max_terms);

// Two functions sampled together (f(r, &f1, &f2)); both truncated to the same length.
void fit_chebyshev_pair(const std::function<void(double, double*, double*)>& f, double lo, double hi, int nodes,
                        double rel_tol, int max_terms, std::vector<double>& c1, std::vector<double>& c2);

// Relative truncation of the FP32 tables' Chebyshev series.  The tables are
// evaluated in FP32 from an FP32 argument, whose rounding alone gives 1-5e-7
// of max |T| near the steep end of the far piece; truncating at 2e-8
// instead of 1e-9 leaves that error unchanged and drops two to three terms
// of the far polynomial (20 -> 17 for most instances).
constexpr double kTableTol = 2e-8;
// Far-polynomial length of the serving slots' kernel; longer fits whose extra
// terms are negligible are cut to it (build_tables).
constexpr int kPreferredTerms = 18;

// Fill the per-instance real-space tables.  poly_tol: relative truncation of
// the Chebyshev series (kTableTol; 1e-9 keeps ~20 terms); max_terms caps the screened
// polynomial (<= 0: kMaxPoly); fp64_far: also fit the FP64 far series of
// the FP64 path (nf = 0 otherwise).  Returns 0 or an error code.
int build_tables(double a, double d, double eps, double rc, double poly_tol, PbTables* t, int max_terms = 0,
                 bool fp64_far = true);

}  // namespace pb
