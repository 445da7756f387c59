/*
 * C entry points over the reference's own host code, for fixture
 * generation only (TEST INFRASTRUCTURE).  Compiled by oracle/build_ref.sh
 * against the reference sources where they lie, never shipped.
 */
#include "periodicBrinkman.h"

extern "C" {
void ref_singH(double r2, double a, double *H) { singH(r2, a, H[0], H[1]); }
void ref_regH(double r2, double a, double d, double *H) { regH(r2, a, d, H[0], H[1]); }
void ref_diffH(double r2, double a, double d, double *H) { diffH(r2, a, d, H[0], H[1]); }
double ref_experf(double x, double z, double c) { return experf(x, z, c); }
void ref_vR(double *A, const double *xh, double a, double d, double e) { vR(A, xh, a, d, e); }
void ref_vF(double *A, const double *xh, double a, double d, const double *k) { vF(A, xh, a, d, k); }

/* A (3m x 3n column-major) from realShells (l = 0, then shells up to Mx)
 * and fourierShells (up to Nx), both starting from oldM = 0, exactly as
 * the reference's driver calls them (cuda/periodicBrinkman.cu:176-182). */
void ref_shells(double *Aout, const double *x, int m, const double *x0, int n, const int *Mx,
                const int *Nx, const double *L, double a, double d, double e)
{
    MatrixOnHost X(3, m), X0(3, n), A(3 * m, 3 * n), absA(3 * m, 3 * n);
    for (int i = 0; i < 3 * m; i++) X(i) = x[i];
    for (int i = 0; i < 3 * n; i++) X0(i) = x0[i];
    MatrixOnHost Lm(3), newM(3), oldM(3);
    for (int q = 0; q < 3; q++) Lm(q) = L[q];
    realShells(A, absA, X, X0, newM, oldM, Lm, a, d, e);
    for (int q = 0; q < 3; q++) newM(q) = Mx[q];
    realShells(A, absA, X, X0, newM, oldM, Lm, a, d, e);
    for (int q = 0; q < 3; q++) newM(q) = Nx[q];
    fourierShells(A, absA, X, X0, newM, oldM, Lm, a, d, e);
    for (int i = 0; i < 9 * m * n; i++) Aout[i] = A.data()[i];
}
}
