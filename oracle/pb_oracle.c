/*
 * pb_oracle.c -- FP64 CPU oracle for the periodic regularized Brinkman hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; it is used by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py, always as the checker and never as the thing
 * measured or shipped.
 *
 * It restates, in plain C and double precision, the algorithm of the
 * reference project hoangngan82/periodicBrinkman:
 *
 *   - the scalar kernel functions experf/singH/regH/diffH and the pair
 *     tensors vR/vF                      (cuda/periodicBrinkman.h:19-208)
 *   - the dense direct-Ewald mobility matrix by real and Fourier shells,
 *     including the per-axis shell counts of periodicBrinkman()
 *                                         (cuda/periodicBrinkman.h:432-513,
 *                                          cuda/periodicBrinkman.h:564-823)
 *   - the velocity u = sum_j A(x_i - x_j) f_j of the spectral-Ewald entry
 *     point, written as a converged direct Ewald sum: real space over
 *     periodic images found with a cell list, k space through the
 *     structure factor with the modified-blob symbol of the reference
 *     (cuda/periodicBrinkman.h:183-208, cuda/fftBrinkman.h:179-219), the
 *     k = 0 mode dropped (cuda/fftBrinkman.h:201-207) unless asked for.
 *
 * Two evaluators of the real-space pair kernel are provided:
 *   "faithful": the reference's closed forms verbatim in structure, with a
 *               switch radius (the reference's `eps`) below which the r -> 0
 *               limit is used (cuda/periodicBrinkman.h:95,105-111);
 *   "accurate": the same closed forms where they are well conditioned, and
 *               for r < 0.2*delta the regularized Brinkmanlet from its radial
 *               Fourier integral (Gauss-Legendre), which has no r -> 0
 *               cancellation.
 *
 * Parity of this oracle is pinned against fixtures generated from the
 * reference's own host code (tests/golden/, see oracle/build_ref.sh) and
 * against 50-digit mpmath values of the Fourier-integral definition.
 *
 * Layout conventions follow the reference: a 3 x N column-major matrix is an
 * array of N xyz triples; the mobility matrix A is 3m x 3n column-major with
 * A(3*i + r, 3*j + c) the (r, c) entry of the block of target i and source j
 * (cuda/periodicBrinkman.h:16-17, 304).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PBO_PI  3.14159265358979323846264338327950288
#define PBO_SPI 1.77245385090551602729816748334114518 /* sqrt(pi) */
#define IDX2D(row, col) (((col) * 3) + (row))

static double g_eps_switch = 1e-12;

void pbo_set_eps_switch(double e) { g_eps_switch = e; }
double pbo_get_eps_switch(void) { return g_eps_switch; }

int pbo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void pbo_set_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------ */
/* Faithful scalar functions (cuda/periodicBrinkman.h:19-208)          */
/* ------------------------------------------------------------------ */

/* exp(c*x*z) * erfc(z + x), zero when both |x|, |z| are large and x*z >= 0
 * (cuda/periodicBrinkman.h:19-25). */
double pbo_experf(double x, double z, double c)
{
    double a = 0;
    if ((x * z < 0) || (x * x + z * z < 700)) a = exp(c * x * z) * erfc(z + x);
    return a;
}

/* Singular Brinkmanlet H1, H2 (cuda/periodicBrinkman.h:31-46). */
void pbo_singH(double r2, double a, double *H1, double *H2)
{
    double r = sqrt(r2);
    if (r > g_eps_switch) {
        *H1 = -1 / (4 * PBO_PI * a * a * r * r2) +
              exp(-a * r) / (4 * PBO_PI * r) * (1 + 1 / (a * r) + 1 / (a * a * r2));
        *H2 = 3 / (4 * PBO_PI * a * a * r * r2 * r2) -
              exp(-a * r) / (4 * PBO_PI * r2 * r) * (1 + 3 / (a * r) + 3 / (a * a * r2));
    } else {
        *H1 = *H2 = 1.79e+308;
    }
}

/* Regularized Brinkmanlet R_d: H1, H2 (cuda/periodicBrinkman.h:53-78). */
void pbo_regH(double r2, double a, double d, double *H1, double *H2)
{
    double expx2 = exp(-r2 / d / d);
    double r = sqrt(r2);
    double Erf = erf(r / d);
    double c = 1 - exp(-a * a * d * d / 4);
    if (r > g_eps_switch) {
        double h1 = -1 / (4 * PBO_PI * a * a * r2 * r) * Erf;
        h1 += 1 / (2 * a * a * d * d * d * PBO_PI * PBO_SPI * r2) * expx2 * (d * d + 2 * r2) * c;
        h1 += 1 / (8 * a * a * PBO_PI * r2 * r) * (1 + a * r + a * a * r2) * pbo_experf(a * d / 2, -r / d, 2);
        h1 -= 1 / (8 * a * a * PBO_PI * r2 * r) * (1 - a * r + a * a * r2) * pbo_experf(a * d / 2, r / d, 2);
        double h2 = 3 / (4 * PBO_PI * a * a * r2 * r2 * r) * Erf;
        h2 -= c / (2 * a * a * d * d * d * PBO_PI * PBO_SPI * r2 * r2) * expx2 * (3 * d * d + 2 * r2);
        h2 -= 1 / (8 * a * a * PBO_PI * r2 * r2 * r) * (3 + 3 * a * r + a * a * r2) * pbo_experf(a * d / 2, -r / d, 2);
        h2 += 1 / (8 * a * a * PBO_PI * r2 * r2 * r) * (3 - 3 * a * r + a * a * r2) * pbo_experf(a * d / 2, r / d, 2);
        *H1 = h1;
        *H2 = h2;
    } else {
        double x = a * a * d * d;
        *H1 = -a * erfc(a * d / 2) / (6 * PBO_PI) + (2 + exp(-x / 4) * (x - 2)) / (3 * a * a * d * d * d * PBO_PI * PBO_SPI);
        double h2 = (-24 + 2 * x * (2 - x)) * exp(-x / 4) + 24;
        *H2 = h2 / (60 * a * a * d * d * d * d * d * PBO_PI * PBO_SPI) + a * a * a / (60 * PBO_PI) * erfc(a * d / 2);
    }
}

/* Singular minus regularized: diffH = S - R_d (cuda/periodicBrinkman.h:85-112).
 * For r at or below the switch radius the r -> 0 limit -R_d(0) is returned. */
void pbo_diffH(double r2, double a, double d, double *dH1, double *dH2)
{
    double expx2 = exp(-r2 / d / d) * (1 - exp(-a * a * d * d / 4));
    double r = sqrt(r2);
    double Erfc = erfc(r / d);
    if (r > g_eps_switch) {
        double h1 = -1 / (4 * PBO_PI * a * a) / (r2 * r) * Erfc;
        h1 -= (d * d + 2 * r2) / (2 * a * a * d * d * d * PBO_PI * PBO_SPI * r2) * expx2;
        h1 += 1 / (8 * PBO_PI * a * a * r2 * r) * (1 + a * r + a * a * r2) * pbo_experf(-a * d / 2, r / d, 2);
        h1 += 1 / (8 * PBO_PI * a * a * r2 * r) * (1 - a * r + a * a * r2) * pbo_experf(a * d / 2, r / d, 2);
        double h2 = 3 / (4 * PBO_PI * a * a) / (r2 * r2 * r) * Erfc;
        h2 += (3 * d * d + 2 * r2) / (2 * a * a * d * d * d * PBO_PI * PBO_SPI * r2 * r2) * expx2;
        h2 -= 1 / (8 * PBO_PI * a * a * r2 * r2 * r) * (3 + 3 * a * r + a * a * r2) * pbo_experf(-a * d / 2, r / d, 2);
        h2 -= 1 / (8 * PBO_PI * a * a * r2 * r2 * r) * (3 - 3 * a * r + a * a * r2) * pbo_experf(a * d / 2, r / d, 2);
        *dH1 = h1;
        *dH2 = h2;
    } else {
        double x = a * a * d * d;
        *dH1 = -(4 + 2 * (-2 + x) * exp(-x / 4)) / (x * d * 6 * PBO_PI * PBO_SPI) + a * erfc(a * d / 2) / (6 * PBO_PI);
        *dH2 = -(2 - x) * exp(-x / 4) / (30 * d * d * d * PBO_PI * PBO_SPI) -
               2 * (1 - exp(-x / 4)) / (5 * x * d * d * d * PBO_PI * PBO_SPI) -
               a * a * a * erfc(a * d / 2) / (60 * PBO_PI);
    }
}

/* Real-space pair tensor: H = diffH(d) - diffH(e), A = H1 I + H2 x x^T
 * (cuda/periodicBrinkman.h:152-176).  e = 0 means singular point forces. */
void pbo_vR(double *A, const double *xh, double a, double d, double e)
{
    double H1, H2, tH1 = 0, tH2 = 0;
    double r2 = xh[0] * xh[0] + xh[1] * xh[1] + xh[2] * xh[2];
    pbo_diffH(r2, a, d, &H1, &H2);
    if (e > 0) pbo_diffH(r2, a, e, &tH1, &tH2);
    H1 -= tH1;
    H2 -= tH2;
    for (int i = 0; i < 3; i++) {
        for (int j = 0; j < 3; j++) A[IDX2D(i, j)] = xh[i] * xh[j] * H2;
        A[IDX2D(i, i)] += H1;
    }
}

/* k-space pair tensor (k^2 I - k k^T) bhat cos(k.x) with the modified-blob
 * symbol (cuda/periodicBrinkman.h:183-208).  Not divided by the cell volume. */
void pbo_vF(double *A, const double *xh, double a, double d, const double *k)
{
    double kx = xh[0] * k[0] + xh[1] * k[1] + xh[2] * k[2];
    double kn = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
    double x = a * d * a * d;
    double w = d * d * kn;
    double a1 = 1 - exp(-x / 4);
    double a0 = x + 6 * a1;
    double bhat = 1 / x * (a1 * (w - 6) + a0) * exp(-w / 4) * cos(kx);
    bhat *= 1 / (kn * (kn + a * a));
    for (int i = 0; i < 3; i++) {
        A[IDX2D(i, i)] = 0;
        for (int j = 0; j < 3; j++) {
            if (i != j) {
                A[IDX2D(i, j)] = -k[i] * k[j] * bhat;
                A[IDX2D(i, i)] += k[j] * k[j] * bhat;
            }
        }
    }
}

/* Fourier symbol of the splitting blob (the bracket of cuda/fftBrinkman.h:196
 * and cuda/periodicBrinkman.h:191-195): [1 + (1 - e^{-a^2 d^2/4}) k^2/a^2] e^{-k^2 d^2/4}. */
double pbo_phihat(double kn, double a, double d)
{
    double x = a * a * d * d;
    double a1 = -expm1(-x / 4);
    return (1.0 + a1 * kn / (a * a)) * exp(-d * d * kn / 4);
}

/* ------------------------------------------------------------------ */
/* Per-axis shell counts of periodicBrinkman() (P.h:457-487)           */
/* ------------------------------------------------------------------ */
void pbo_shell_counts(const double *L, int M, int N, int *Mx, int *Nx)
{
    int idL[3] = {0, 1, 2};
    int temp;
    Mx[0] = Mx[1] = Mx[2] = M;
    Nx[0] = Nx[1] = Nx[2] = N;
    if (L[idL[0]] > L[idL[1]]) {
        temp = idL[0]; idL[0] = idL[1]; idL[1] = temp;
    }
    if (L[idL[2]] <= L[idL[0]]) {
        temp = idL[2]; idL[2] = idL[1]; idL[1] = idL[0]; idL[0] = temp;
    } else if (L[idL[2]] < L[idL[1]]) {
        temp = idL[1]; idL[1] = idL[2]; idL[2] = temp;
    }
    Mx[idL[2]] = (int)ceil(M * L[idL[0]] / L[idL[2]]);
    Mx[idL[1]] = (int)ceil(M * L[idL[0]] / L[idL[1]]);
    Nx[idL[0]] = (int)ceil(N * L[idL[2]] / L[idL[0]]);
    Nx[idL[1]] = (int)ceil(N * L[idL[2]] / L[idL[1]]);
}

/* ------------------------------------------------------------------ */
/* Dense mobility matrix by shells (faithful)                          */
/* ------------------------------------------------------------------ */
static void add_block(double *A, long lda, int i, int j, const double *t, double scale)
{
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) A[(long)(3 * j + c) * lda + 3 * i + r] += t[IDX2D(r, c)] * scale;
}

/* A(3m x 3n, column-major) = sum over real images l in the box
 * [-Mx,Mx]x[-My,My]x[-Mz,Mz] of vR(x_i - x0_j - l*L)
 * + (1/tau) sum over k = 2 pi n / L, n in [-Nx,Nx]x.. minus 0, of vF.
 * The image and wave-vector boxes are walked in the face order of
 * realShells / fourierShells (cuda/periodicBrinkman.h:578-690, 723-820)
 * starting from oldM = 0.  A is overwritten.  Mx/Nx < 0 skips that part. */
void pbo_shell_matrix(double *A, const double *x, int m, const double *x0, int n,
                      double a, double d, double e, const int *Mx, const int *Nx,
                      const double *L)
{
    long lda = 3L * m;
    memset(A, 0, sizeof(double) * (size_t)lda * 3 * n);
    double tau = L[0] * L[1] * L[2];
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (int i = 0; i < m; i++) {
        for (int j = 0; j < n; j++) {
            double xh0[3], xh[3], t[9];
            for (int k = 0; k < 3; k++) xh0[k] = x[3 * i + k] - x0[3 * j + k];
            if (Mx[0] >= 0) {
                pbo_vR(t, xh0, a, d, e);
                add_block(A, lda, i, j, t, 1.0);
                /* top and bottom faces */
                for (int l3 = 0; l3 < Mx[2]; l3++)
                    for (int l2 = -Mx[1]; l2 <= Mx[1]; l2++)
                        for (int l1 = -Mx[0]; l1 <= Mx[0]; l1++) {
                            xh[2] = xh0[2] - (l3 + 1) * L[2];
                            xh[1] = xh0[1] - l2 * L[1];
                            xh[0] = xh0[0] - l1 * L[0];
                            pbo_vR(t, xh, a, d, e); add_block(A, lda, i, j, t, 1.0);
                            xh[2] = xh0[2] + (l3 + 1) * L[2];
                            pbo_vR(t, xh, a, d, e); add_block(A, lda, i, j, t, 1.0);
                        }
                /* left and right faces */
                for (int l2 = 1; l2 <= Mx[1]; l2++)
                    for (int l1 = -Mx[0]; l1 <= Mx[0]; l1++) {
                        xh[2] = xh0[2];
                        xh[1] = xh0[1] - l2 * L[1];
                        xh[0] = xh0[0] - l1 * L[0];
                        pbo_vR(t, xh, a, d, e); add_block(A, lda, i, j, t, 1.0);
                        xh[1] = xh0[1] + l2 * L[1];
                        pbo_vR(t, xh, a, d, e); add_block(A, lda, i, j, t, 1.0);
                    }
                /* front and back faces */
                for (int l1 = 1; l1 <= Mx[0]; l1++) {
                    xh[2] = xh0[2];
                    xh[1] = xh0[1];
                    xh[0] = xh0[0] - l1 * L[0];
                    pbo_vR(t, xh, a, d, e); add_block(A, lda, i, j, t, 1.0);
                    xh[0] = xh0[0] + l1 * L[0];
                    pbo_vR(t, xh, a, d, e); add_block(A, lda, i, j, t, 1.0);
                }
            }
            if (Nx[0] > 0 || Nx[1] > 0 || Nx[2] > 0) {
                double kv[3];
                for (int l3 = 1; l3 <= Nx[2]; l3++)
                    for (int l2 = -Nx[1]; l2 <= Nx[1]; l2++)
                        for (int l1 = -Nx[0]; l1 <= Nx[0]; l1++) {
                            kv[0] = 2 * PBO_PI * l1 / L[0];
                            kv[1] = 2 * PBO_PI * l2 / L[1];
                            kv[2] = 2 * PBO_PI * l3 / L[2];
                            pbo_vF(t, xh0, a, d, kv); add_block(A, lda, i, j, t, 1.0 / tau);
                            kv[2] = -kv[2];
                            pbo_vF(t, xh0, a, d, kv); add_block(A, lda, i, j, t, 1.0 / tau);
                        }
                for (int l2 = 1; l2 <= Nx[1]; l2++)
                    for (int l1 = -Nx[0]; l1 <= Nx[0]; l1++) {
                        kv[0] = 2 * PBO_PI * l1 / L[0];
                        kv[1] = 2 * PBO_PI * l2 / L[1];
                        kv[2] = 0;
                        pbo_vF(t, xh0, a, d, kv); add_block(A, lda, i, j, t, 1.0 / tau);
                        kv[1] = -kv[1];
                        pbo_vF(t, xh0, a, d, kv); add_block(A, lda, i, j, t, 1.0 / tau);
                    }
                for (int l1 = 1; l1 <= Nx[0]; l1++) {
                    kv[0] = 2 * PBO_PI * l1 / L[0];
                    kv[1] = 0;
                    kv[2] = 0;
                    pbo_vF(t, xh0, a, d, kv); add_block(A, lda, i, j, t, 1.0 / tau);
                    kv[0] = -kv[0];
                    pbo_vF(t, xh0, a, d, kv); add_block(A, lda, i, j, t, 1.0 / tau);
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Accurate pair kernel                                                */
/* ------------------------------------------------------------------ */

/* Singular Brinkmanlet without the small-alpha*r cancellation:
 * r S1 = A1(u)/(4 pi), r^3 S2 = A2(u)/(4 pi), u = alpha r, with
 * A1 = (-1 + e^{-u}(1+u+u^2))/u^2 and A2 = (3 - e^{-u}(3+3u+u^2))/u^2
 * (the closed forms of cuda/periodicBrinkman.h:41-42), summed as power
 * series below u = 0.5. */
static void stable_S(double r, double a, double *S1, double *S2)
{
    double u = a * r, A1, A2;
    if (u < 0.5) {
        double s1 = 0, s2 = 0, p = 1, fact = 2; /* p = u^{k-2}, fact = k! */
        for (int k = 2; k < 40; k++) {
            double sg = (k & 1) ? -1.0 : 1.0;
            double t1 = sg * (k - 1.0) * (k - 1.0) / fact * p;
            double t2 = -sg * (k - 1.0) * (k - 3.0) / fact * p;
            s1 += t1;
            s2 += t2;
            if (fabs(t1) < 1e-19 * fabs(s1) && fabs(t2) < 1e-19 * fabs(s2) && k > 4) break;
            p *= u;
            fact *= (k + 1);
        }
        A1 = s1;
        A2 = s2;
    } else {
        double em = exp(-u);
        A1 = (-1 + em * (1 + u + u * u)) / (u * u);
        A2 = (3 - em * (3 + 3 * u + u * u)) / (u * u);
    }
    *S1 = A1 / (4 * PBO_PI * r);
    *S2 = A2 / (4 * PBO_PI * r * r * r);
}

/* j0(z) - j1(z)/z and j2(z)/z^2 without cancellation at small z. */
static void sph_combos(double z, double *s1, double *s2)
{
    if (z < 2.0) {
        double z2 = z * z, t1 = 2.0 / 3.0, t2 = 1.0 / 15.0, a1 = 0, a2 = 0;
        for (int m = 0; m < 60; m++) {
            a1 += t1;
            a2 += t2;
            if (fabs(t1) < 1e-19 && fabs(t2) < 1e-19) break;
            t1 *= -z2 * (m + 2.0) * (m + 2.0) / ((m + 1.0) * (m + 1.0) * (2 * m + 4.0) * (2 * m + 5.0));
            t2 *= -z2 / (2.0 * (m + 1.0) * (2 * m + 7.0));
        }
        *s1 = a1;
        *s2 = a2;
    } else {
        double sz = sin(z), cz = cos(z);
        double j0 = sz / z;
        double j1 = sz / (z * z) - cz / z;
        double j2 = (3 / (z * z) - 1) * sz / z - 3 * cz / (z * z);
        *s1 = j0 - j1 / z;
        *s2 = j2 / (z * z);
    }
}

/* 16-point Gauss-Legendre nodes/weights on [-1,1], computed once. */
static double gl_x[16], gl_w[16];
static int gl_ready = 0;
static void gl_init(void)
{
    if (gl_ready) return;
    const int n = 16;
    for (int i = 0; i < n; i++) {
        double x = cos(PBO_PI * (i + 0.75) / (n + 0.5)), dp = 1;
        for (int it = 0; it < 100; it++) {
            double p0 = 1, p1 = x;
            for (int k = 2; k <= n; k++) {
                double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            dp = n * (x * p1 - p0) / (x * x - 1);
            double dx = p1 / dp;
            x -= dx;
            if (fabs(dx) < 1e-17) break;
        }
        gl_x[i] = x;
        gl_w[i] = 2 / ((1 - x * x) * dp * dp);
    }
    gl_ready = 1;
}

static int cmp_dbl(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

/* Regularized Brinkmanlet from its radial Fourier integral:
 *   H1(r) = 1/(2 pi^2) int_0^inf phi(k) k^2/(k^2+a^2) [j0(kr) - j1(kr)/(kr)] dk
 *   H2(r) = 1/(2 pi^2) int_0^inf phi(k) k^4/(k^2+a^2) j2(kr)/(kr)^2 dk
 * with phi = phihat(k; d1) (mode 0) or phihat(k; d1) - phihat(k; d2)
 * (mode 1, i.e. R_d1 - R_d2).  phihat is the modified-blob symbol of
 * cuda/periodicBrinkman.h:189-196. */
void pbo_reg_quad(double r, double a, double d1, double d2, int mode, double *H1, double *H2)
{
    gl_init();
    double dmin = (mode == 1 && d2 < d1) ? d2 : d1;
    double dmax = (mode == 1 && d2 > d1) ? d2 : d1;
    double K = 14.0 / dmin;
    double w = 1.0 / dmin;
    if (r > 0 && 1.5 / r < w) w = 1.5 / r;
    int nu = (int)ceil(K / w);
    double *edges = (double *)malloc(sizeof(double) * (nu + 64));
    int ne = 0;
    for (int i = 0; i <= nu; i++) edges[ne++] = K * i / nu;
    for (int j = -4; j <= 4; j++) {
        double e = a * ldexp(1.0, j);
        if (e > 0 && e < K) edges[ne++] = e;
    }
    /* the wider blob decays on the k scale 1/dmax: resolve it too */
    for (int i = 1; i <= 28; i++) {
        double e = 0.5 * i / dmax;
        if (e < K) edges[ne++] = e;
    }
    qsort(edges, ne, sizeof(double), cmp_dbl);
    double s1 = 0, s2 = 0;
    for (int p = 0; p + 1 < ne; p++) {
        double lo = edges[p], hi = edges[p + 1];
        if (hi - lo < 1e-14 * K) continue;
        double c = 0.5 * (lo + hi), h = 0.5 * (hi - lo);
        for (int q = 0; q < 16; q++) {
            double k = c + h * gl_x[q], kn = k * k;
            double ph = pbo_phihat(kn, a, d1);
            if (mode == 1) ph -= pbo_phihat(kn, a, d2);
            double b1, b2;
            sph_combos(k * r, &b1, &b2);
            double g = ph * kn / (kn + a * a) * gl_w[q] * h;
            s1 += g * b1;
            s2 += g * kn * b2;
        }
    }
    free(edges);
    *H1 = s1 / (2 * PBO_PI * PBO_PI);
    *H2 = s2 / (2 * PBO_PI * PBO_PI);
}

/* Closed-form diffH without the switch radius (r > 0 assumed). */
static void diffH_closed(double r, double a, double d, double *h1, double *h2)
{
    double sw = g_eps_switch;
    g_eps_switch = -1.0;
    pbo_diffH(r * r, a, d, h1, h2);
    g_eps_switch = sw;
}

/* Accurate real-space pair kernel H = (R_e - R_d) (e > 0) or S - R_d (e = 0):
 *   closed forms of diffH where r >= 0.2 delta (cuda/periodicBrinkman.h:85-112),
 *   the Fourier integral of the regularized part below that, and for the
 *   blob pair also where alpha*r < 0.2 (the closed forms lose ~(alpha r)^-2).
 * At r = 0 with e = 0 it returns the reference's limit -R_d(0)
 * (cuda/periodicBrinkman.h:105-111). */
void pbo_pairH(double r, double a, double d, double e, double *H1, double *H2)
{
    if (e > 0 && (r < 0.2 * e || ((r < 0.2 * d || a * r < 0.2) && r < 9 * e))) {
        pbo_reg_quad(r, a, e, d, 1, H1, H2);
        return;
    }
    double hd1, hd2, he1 = 0, he2 = 0;
    if (r < 0.2 * d) {
        double R1, R2;
        pbo_reg_quad(r, a, d, d, 0, &R1, &R2);
        if (r == 0) {
            hd1 = -R1;
            hd2 = -R2;
        } else {
            double S1, S2;
            stable_S(r, a, &S1, &S2);
            hd1 = S1 - R1;
            hd2 = S2 - R2;
        }
    } else {
        diffH_closed(r, a, d, &hd1, &hd2);
    }
    if (e > 0 && r < 9 * e) diffH_closed(r, a, e, &he1, &he2);
    *H1 = hd1 - he1;
    *H2 = hd2 - he2;
}

/* ------------------------------------------------------------------ */
/* Converged direct Ewald sum for velocities                           */
/* ------------------------------------------------------------------ */

#define PBO_REAL 1
#define PBO_KSPACE 2
#define PBO_ZERO_MODE 4

static double wrap1(double v, double L)
{
    double w = v - L * floor(v / L);
    if (w >= L) w -= L;
    if (w < 0) w = 0;
    return w;
}

/* U (m x 3) = velocities at targets y (m x 3) induced by forces f at
 * sources x (n x 3) in the periodic box L, Brinkman alpha a, blob e,
 * Ewald splitting blob d.  rc <= 0 / kc <= 0 choose converged cutoffs
 * (6 d and 14 / d).  flags: PBO_REAL | PBO_KSPACE | PBO_ZERO_MODE.
 * Returns 0, or -1 on bad input / allocation failure. */
int pbo_ewald_velocity(double *U, const double *y, int m, const double *x, const double *f, int n,
                       const double *L, double a, double e, double d, double rc, double kc, int flags)
{
    if (m < 0 || n < 0 || !(L[0] > 0 && L[1] > 0 && L[2] > 0) || !(a > 0) || !(d > 0) || e < 0) return -1;
    if (rc <= 0) rc = 6.0 * d;
    if (kc <= 0) kc = 14.0 / d;
    double tau = L[0] * L[1] * L[2];
    memset(U, 0, sizeof(double) * 3 * (size_t)m);
    if (m == 0 || n == 0) return 0;

    if (flags & PBO_REAL) {
        int nc[3], S[3];
        double h[3];
        for (int q = 0; q < 3; q++) {
            nc[q] = (int)floor(L[q] / rc);
            if (nc[q] < 1) nc[q] = 1;
            if (nc[q] > 64) nc[q] = 64;
            h[q] = L[q] / nc[q];
            S[q] = (int)ceil(rc / h[q]);
        }
        long ncell = (long)nc[0] * nc[1] * nc[2];
        int *start = (int *)calloc(ncell + 1, sizeof(int));
        int *order = (int *)malloc(sizeof(int) * (size_t)n);
        double *xs = (double *)malloc(sizeof(double) * 3 * (size_t)n);
        int *cell = (int *)malloc(sizeof(int) * (size_t)n);
        if (!start || !order || !xs || !cell) {
            free(start); free(order); free(xs); free(cell);
            return -1;
        }
        for (int j = 0; j < n; j++) {
            int ci[3];
            for (int q = 0; q < 3; q++) {
                xs[3 * j + q] = wrap1(x[3 * j + q], L[q]);
                ci[q] = (int)(xs[3 * j + q] / h[q]);
                if (ci[q] >= nc[q]) ci[q] = nc[q] - 1;
            }
            cell[j] = (ci[0] * nc[1] + ci[1]) * nc[2] + ci[2];
            start[cell[j] + 1]++;
        }
        for (long c = 0; c < ncell; c++) start[c + 1] += start[c];
        int *fill = (int *)malloc(sizeof(int) * (size_t)ncell);
        memcpy(fill, start, sizeof(int) * (size_t)ncell);
        for (int j = 0; j < n; j++) order[fill[cell[j]]++] = j;
        free(fill);
        double rc2 = rc * rc;
#pragma omp parallel for schedule(dynamic, 16)
        for (int i = 0; i < m; i++) {
            double yt[3];
            int ct[3];
            for (int q = 0; q < 3; q++) {
                yt[q] = wrap1(y[3 * i + q], L[q]);
                ct[q] = (int)(yt[q] / h[q]);
                if (ct[q] >= nc[q]) ct[q] = nc[q] - 1;
            }
            double u0 = 0, u1 = 0, u2 = 0;
            for (int o0 = -S[0]; o0 <= S[0]; o0++) {
                int g0 = ct[0] + o0;
                int c0 = ((g0 % nc[0]) + nc[0]) % nc[0];
                double sh0 = (double)((g0 - c0) / nc[0]) * L[0];
                for (int o1 = -S[1]; o1 <= S[1]; o1++) {
                    int g1 = ct[1] + o1;
                    int c1 = ((g1 % nc[1]) + nc[1]) % nc[1];
                    double sh1 = (double)((g1 - c1) / nc[1]) * L[1];
                    for (int o2 = -S[2]; o2 <= S[2]; o2++) {
                        int g2 = ct[2] + o2;
                        int c2 = ((g2 % nc[2]) + nc[2]) % nc[2];
                        double sh2 = (double)((g2 - c2) / nc[2]) * L[2];
                        long cs = ((long)c0 * nc[1] + c1) * nc[2] + c2;
                        for (int p = start[cs]; p < start[cs + 1]; p++) {
                            int j = order[p];
                            double dx = yt[0] - (xs[3 * j] + sh0);
                            double dy = yt[1] - (xs[3 * j + 1] + sh1);
                            double dz = yt[2] - (xs[3 * j + 2] + sh2);
                            double r2 = dx * dx + dy * dy + dz * dz;
                            if (r2 >= rc2) continue;
                            double H1, H2;
                            pbo_pairH(sqrt(r2), a, d, e, &H1, &H2);
                            double fd = f[3 * j] * dx + f[3 * j + 1] * dy + f[3 * j + 2] * dz;
                            u0 += H1 * f[3 * j] + H2 * fd * dx;
                            u1 += H1 * f[3 * j + 1] + H2 * fd * dy;
                            u2 += H1 * f[3 * j + 2] + H2 * fd * dz;
                        }
                    }
                }
            }
            U[3 * i] += u0;
            U[3 * i + 1] += u1;
            U[3 * i + 2] += u2;
        }
        free(start); free(order); free(xs); free(cell);
    }

    if (flags & PBO_KSPACE) {
        int nm[3];
        for (int q = 0; q < 3; q++) nm[q] = (int)floor(kc * L[q] / (2 * PBO_PI));
        int NY = 2 * nm[1] + 1, NZ = 2 * nm[2] + 1;
        long plane = (long)NY * NZ;
        long nk = (long)(nm[0] + 1) * plane;
        double *W = (double *)calloc((size_t)nk * 6, sizeof(double)); /* re/im x 3 */
        if (!W) return -1;
        double kc2 = kc * kc;
        /* structure factor S(k) = sum_j f_j e^{-i k.x_j}, half space n_x >= 0 */
#pragma omp parallel
        {
            double *ey = (double *)malloc(sizeof(double) * 2 * NY);
            double *ez = (double *)malloc(sizeof(double) * 2 * NZ);
#pragma omp for schedule(dynamic, 1)
            for (int px = 0; px <= nm[0]; px++) {
                double *Wp = W + (long)px * plane * 6;
                for (int j = 0; j < n; j++) {
                    double ax = -2 * PBO_PI * px * x[3 * j] / L[0];
                    double exr = cos(ax), exi = sin(ax);
                    for (int t = -nm[1]; t <= nm[1]; t++) {
                        double ang = -2 * PBO_PI * t * x[3 * j + 1] / L[1];
                        ey[2 * (t + nm[1])] = cos(ang);
                        ey[2 * (t + nm[1]) + 1] = sin(ang);
                    }
                    for (int t = -nm[2]; t <= nm[2]; t++) {
                        double ang = -2 * PBO_PI * t * x[3 * j + 2] / L[2];
                        ez[2 * (t + nm[2])] = cos(ang);
                        ez[2 * (t + nm[2]) + 1] = sin(ang);
                    }
                    double f0 = f[3 * j], f1 = f[3 * j + 1], f2 = f[3 * j + 2];
                    for (int iy = 0; iy < NY; iy++) {
                        double xyr = exr * ey[2 * iy] - exi * ey[2 * iy + 1];
                        double xyi = exr * ey[2 * iy + 1] + exi * ey[2 * iy];
                        double *Wr = Wp + (long)iy * NZ * 6;
                        for (int iz = 0; iz < NZ; iz++) {
                            double er = xyr * ez[2 * iz] - xyi * ez[2 * iz + 1];
                            double ei = xyr * ez[2 * iz + 1] + xyi * ez[2 * iz];
                            double *w6 = Wr + iz * 6;
                            w6[0] += f0 * er; w6[1] += f0 * ei;
                            w6[2] += f1 * er; w6[3] += f1 * ei;
                            w6[4] += f2 * er; w6[5] += f2 * ei;
                        }
                    }
                }
                /* W(k) = (2/tau) Ghat_d(k) S(k), zero outside |k| <= kc and at k = 0 */
                for (int iy = 0; iy < NY; iy++) {
                    for (int iz = 0; iz < NZ; iz++) {
                        int ty = iy - nm[1], tz = iz - nm[2];
                        double *w6 = Wp + ((long)iy * NZ + iz) * 6;
                        int half = (px > 0) || (px == 0 && ty > 0) || (px == 0 && ty == 0 && tz > 0);
                        double k0 = 2 * PBO_PI * px / L[0], k1 = 2 * PBO_PI * ty / L[1], k2 = 2 * PBO_PI * tz / L[2];
                        double kn = k0 * k0 + k1 * k1 + k2 * k2;
                        if (!half || kn > kc2) {
                            for (int q = 0; q < 6; q++) w6[q] = 0;
                            continue;
                        }
                        double b = 2.0 / tau * pbo_phihat(kn, a, d) / (kn * (kn + a * a));
                        for (int ri = 0; ri < 2; ri++) {
                            double v0 = w6[ri], v1 = w6[2 + ri], v2 = w6[4 + ri];
                            double kv = k0 * v0 + k1 * v1 + k2 * v2;
                            w6[ri] = b * (kn * v0 - k0 * kv);
                            w6[2 + ri] = b * (kn * v1 - k1 * kv);
                            w6[4 + ri] = b * (kn * v2 - k2 * kv);
                        }
                    }
                }
            }
            free(ey);
            free(ez);
        }
        /* u(y) += sum_k Re[e^{i k.y} W(k)] */
#pragma omp parallel
        {
            double *ey = (double *)malloc(sizeof(double) * 2 * NY);
            double *ez = (double *)malloc(sizeof(double) * 2 * NZ);
#pragma omp for schedule(dynamic, 16)
            for (int i = 0; i < m; i++) {
                for (int t = -nm[1]; t <= nm[1]; t++) {
                    double ang = 2 * PBO_PI * t * y[3 * i + 1] / L[1];
                    ey[2 * (t + nm[1])] = cos(ang);
                    ey[2 * (t + nm[1]) + 1] = sin(ang);
                }
                for (int t = -nm[2]; t <= nm[2]; t++) {
                    double ang = 2 * PBO_PI * t * y[3 * i + 2] / L[2];
                    ez[2 * (t + nm[2])] = cos(ang);
                    ez[2 * (t + nm[2]) + 1] = sin(ang);
                }
                double u0 = 0, u1 = 0, u2 = 0;
                for (int px = 0; px <= nm[0]; px++) {
                    double ax = 2 * PBO_PI * px * y[3 * i] / L[0];
                    double exr = cos(ax), exi = sin(ax);
                    const double *Wp = W + (long)px * plane * 6;
                    for (int iy = 0; iy < NY; iy++) {
                        double xyr = exr * ey[2 * iy] - exi * ey[2 * iy + 1];
                        double xyi = exr * ey[2 * iy + 1] + exi * ey[2 * iy];
                        const double *Wr = Wp + (long)iy * NZ * 6;
                        for (int iz = 0; iz < NZ; iz++) {
                            double er = xyr * ez[2 * iz] - xyi * ez[2 * iz + 1];
                            double ei = xyr * ez[2 * iz + 1] + xyi * ez[2 * iz];
                            const double *w6 = Wr + iz * 6;
                            u0 += er * w6[0] - ei * w6[1];
                            u1 += er * w6[2] - ei * w6[3];
                            u2 += er * w6[4] - ei * w6[5];
                        }
                    }
                }
                U[3 * i] += u0;
                U[3 * i + 1] += u1;
                U[3 * i + 2] += u2;
            }
            free(ey);
            free(ez);
        }
        free(W);
    }

    if (flags & PBO_ZERO_MODE) {
        double F[3] = {0, 0, 0};
        for (int j = 0; j < n; j++)
            for (int q = 0; q < 3; q++) F[q] += f[3 * j + q];
        for (int i = 0; i < m; i++)
            for (int q = 0; q < 3; q++) U[3 * i + q] += F[q] / (a * a * tau);
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* Free-space Brinkmanlet (no periodicity)                             */
/* ------------------------------------------------------------------ */

/* The reference's Brinkmanlet(A, xh, a, d) (cuda/periodicBrinkman.h:119-141):
 * A = H1 I + H2 xh xh^T with regH (d > 0) or singH (d = 0), the faithful
 * closed forms with the switch radius; A is 3x3 column-major. */
void pbo_brinkmanlet(double *A, const double *xh, double a, double d)
{
    double H1, H2, r2 = xh[0] * xh[0] + xh[1] * xh[1] + xh[2] * xh[2];
    if (d > 0)
        pbo_regH(r2, a, d, &H1, &H2);
    else
        pbo_singH(r2, a, &H1, &H2);
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) A[3 * j + i] = xh[i] * xh[j] * H2 + (i == j ? H1 : 0.0);
}

/* Accurate free-space kernel: R_e (e > 0) from its Fourier integral where
 * r < 0.2 e or alpha r < 0.2 (the closed forms cancel there), else the
 * closed forms of regH; S (e = 0) without the small-alpha r cancellation. */
static void free_pairH(double r, double a, double e, double *H1, double *H2)
{
    if (e > 0) {
        if (r < 0.2 * e || (a * r < 0.2 && r < 9 * e)) {
            pbo_reg_quad(r, a, e, e, 0, H1, H2);
            return;
        }
        double sw = g_eps_switch;
        g_eps_switch = -1.0;
        pbo_regH(r * r, a, e, H1, H2);
        g_eps_switch = sw;
        return;
    }
    stable_S(r, a, H1, H2);
}

/* Free-space velocities u_i = sum_j (H1 I + H2 x x^T) f_j, x = y_i - x_j,
 * with the accurate kernel; for e = 0, coincident pairs (r <= 1e-12) are
 * skipped (no finite velocity).  OpenMP over targets. */
void pbo_brinkmanlet_velocity(double *U, const double *y, int m, const double *x, const double *f, int n,
                              double a, double e)
{
#pragma omp parallel for schedule(dynamic, 4)
    for (int i = 0; i < m; i++) {
        double u0 = 0, u1 = 0, u2 = 0;
        for (int j = 0; j < n; j++) {
            double dx = y[3 * i] - x[3 * j], dy = y[3 * i + 1] - x[3 * j + 1], dz = y[3 * i + 2] - x[3 * j + 2];
            double r = sqrt(dx * dx + dy * dy + dz * dz), H1, H2;
            if (e == 0 && r <= 1e-12) continue;
            free_pairH(r, a, e, &H1, &H2);
            double g = H2 * (f[3 * j] * dx + f[3 * j + 1] * dy + f[3 * j + 2] * dz);
            u0 += H1 * f[3 * j] + g * dx;
            u1 += H1 * f[3 * j + 1] + g * dy;
            u2 += H1 * f[3 * j + 2] + g * dz;
        }
        U[3 * i] = u0;
        U[3 * i + 1] = u1;
        U[3 * i + 2] = u2;
    }
}
