// Dense periodic mobility matrix, the drop-in for the reference's
// periodicBrinkman() (cuda/periodicBrinkman.h:432-513): for every target i
// and source j,
//   A_ij += sum_{l in box(Mx,My,Mz)} vR(x_i - x0_j - l*L)
//         + (1/tau) sum_{n in box(Nx,Ny,Nz), n != 0} vF(x_i - x0_j, 2 pi n / L)
// in FP64 with the reference's per-axis shell counts.  One warp per (i, j)
// pair; lanes stride over images and wave vectors, the nine tensor sums are
// reduced with warp shuffles.  The phase e^{i k.x} is built from per-axis
// tables e^{i l theta_a} held in shared memory; the pair-independent factor
// of each wave vector (its Gaussian, the Brinkman denominator and 1/tau) is
// computed once per block into a shared tile that all the block's pairs read.
#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

constexpr int kDenseWarps = 8;
constexpr int kDenseMaxN = 256;  // max Fourier shells per axis
constexpr int kDenseKT = 512;    // wave vectors per shared tile

struct DenseArgs {
    double a, d, e, c_d, c_e, tau_inv;
    double L[3];
    int Mx[3], Nx[3];
    int m, n;
};

__global__ void __launch_bounds__(kDenseWarps * 32)
    k_dense(double* __restrict__ dA, const double* __restrict__ dx, const double* __restrict__ dx0, DenseArgs A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int tab_len = (2 * A.Nx[0] + 1) + (2 * A.Nx[1] + 1) + (2 * A.Nx[2] + 1);
    // per wave vector of the tile: its factor times the six entries of
    // k^2 I - k k^T (xx, yy, zz, xy, xz, yz), and its shell indices (10 bits each)
    double2* kg = (double2*)smem_raw;                    // [3][kDenseKT]
    int* kl = (int*)(kg + 3 * kDenseKT);                 // [kDenseKT]
    double2* tab = (double2*)(kl + kDenseKT) + (size_t)w * tab_len;
    long long pair = (long long)blockIdx.x * kDenseWarps + w;
    // warps past the last pair still take part in the block's k tiles
    const bool live = pair < (long long)A.m * A.n;
    if (!live) pair = 0;
    const int i = (int)(pair % A.m), j = (int)(pair / A.m);
    double xh0[3];
    for (int q = 0; q < 3; q++) xh0[q] = dx[3 * (size_t)i + q] - dx0[3 * (size_t)j + q];
    double s[6] = {0, 0, 0, 0, 0, 0};  // xx, yy, zz, xy, xz, yz

    // real-space images (cuda/periodicBrinkman.h:265-282)
    const int n0 = 2 * A.Mx[0] + 1, n1 = 2 * A.Mx[1] + 1, n2 = 2 * A.Mx[2] + 1;
    const int nimg = (A.Mx[0] >= 0) ? n0 * n1 * n2 : 0;
    for (int t = lane; t < (live ? nimg : 0); t += 32) {
        int l1 = t % n0 - A.Mx[0];
        int l2 = (t / n0) % n1 - A.Mx[1];
        int l3 = t / (n0 * n1) - A.Mx[2];
        double x0 = xh0[0] - l1 * A.L[0], x1 = xh0[1] - l2 * A.L[1], x2 = xh0[2] - l3 * A.L[2];
        double r2 = x0 * x0 + x1 * x1 + x2 * x2;
        double r = sqrt(r2);
        double H1, H2;
        if (r > 1e-12) {
            diffH_d(r, A.a, A.d, A.c_d, H1, H2);
            if (A.e > 0) {
                double e1, e2;
                diffH_d(r, A.a, A.e, A.c_e, e1, e2);
                H1 -= e1;
                H2 -= e2;
            }
        } else {
            // r -> 0 limits of diffH (cuda/periodicBrinkman.h:105-111)
            const double kSqrtPi = 1.77245385090551602729816748334114518;
            auto lim1 = [&](double dd, double cc) {
                double x = A.a * A.a * dd * dd;
                return -(4 + 2 * (-2 + x) * exp(-x / 4)) / (x * dd * 6 * kPiD * kSqrtPi) +
                       A.a * erfc(A.a * dd / 2) / (6 * kPiD);
            };
            H1 = lim1(A.d, A.c_d) - (A.e > 0 ? lim1(A.e, A.c_e) : 0.0);
            H2 = 0;  // multiplies x x^T = 0
        }
        s[0] += H1 + H2 * x0 * x0;
        s[1] += H1 + H2 * x1 * x1;
        s[2] += H1 + H2 * x2 * x2;
        s[3] += H2 * x0 * x1;
        s[4] += H2 * x0 * x2;
        s[5] += H2 * x1 * x2;
    }

    // k space (cuda/periodicBrinkman.h:371-393 and 739-745, with 1/tau)
    const int N0 = A.Nx[0], N1 = A.Nx[1], N2 = A.Nx[2];
    if (N0 > 0 || N1 > 0 || N2 > 0) {
        double2* t0 = tab;
        double2* t1 = tab + (2 * N0 + 1);
        double2* t2 = t1 + (2 * N1 + 1);
        for (int q = lane; q < tab_len; q += 32) {
            int ax, l;
            if (q < 2 * N0 + 1) {
                ax = 0;
                l = q - N0;
            } else if (q < 2 * N0 + 2 * N1 + 2) {
                ax = 1;
                l = q - (2 * N0 + 1) - N1;
            } else {
                ax = 2;
                l = q - (2 * N0 + 2 * N1 + 2) - N2;
            }
            double sv, cv;
            sincospi(2.0 * l * xh0[ax] / A.L[ax], &sv, &cv);
            (ax == 0 ? t0 : ax == 1 ? t1 : t2)[l + (ax == 0 ? N0 : ax == 1 ? N1 : N2)] = make_double2(cv, sv);
        }
        __syncwarp();
        const double x = A.a * A.d * A.a * A.d;
        const double a1 = -expm1(-x / 4), a0 = x + 6 * a1;
        const long long m0 = 2 * N0 + 1, m1 = 2 * N1 + 1, m2 = 2 * N2 + 1;
        const long long nk = m0 * m1 * m2;
        const double w0 = 2 * kPiD / A.L[0], w1 = 2 * kPiD / A.L[1], w2 = 2 * kPiD / A.L[2];
        for (long long kb = 0; kb < nk; kb += kDenseKT) {
            const int cnt = (int)min((long long)kDenseKT, nk - kb);
            __syncthreads();  // the previous tile is consumed
            for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
                const long long t = kb + q;
                const int l1 = (int)(t % m0) - N0, l2 = (int)((t / m0) % m1) - N1, l3 = (int)(t / (m0 * m1)) - N2;
                const double k0 = w0 * l1, k1 = w1 * l2, k2 = w2 * l3;
                const double kn = k0 * k0 + k1 * k1 + k2 * k2;
                const double wv = A.d * A.d * kn;
                const double g = (l1 == 0 && l2 == 0 && l3 == 0)
                                     ? 0.0
                                     : (a1 * (wv - 6) + a0) * exp(-wv / 4) / (x * kn * (kn + A.a * A.a)) * A.tau_inv;
                kg[q] = make_double2((k1 * k1 + k2 * k2) * g, (k0 * k0 + k2 * k2) * g);
                kg[kDenseKT + q] = make_double2((k0 * k0 + k1 * k1) * g, -k0 * k1 * g);
                kg[2 * kDenseKT + q] = make_double2(-k0 * k2 * g, -k1 * k2 * g);
                kl[q] = (l1 + N0) | ((l2 + N1) << 10) | ((l3 + N2) << 20);
            }
            __syncthreads();
            if (!live) continue;
            for (int q = lane; q < cnt; q += 32) {
                const int pk = kl[q];
                const int i1 = pk & 1023, i2 = (pk >> 10) & 1023, i3 = pk >> 20;
                const double2 e0 = t0[i1], e1 = t1[i2], e2 = t2[i3];
                const double pr = e0.x * e1.x - e0.y * e1.y, pi = e0.x * e1.y + e0.y * e1.x;
                const double cv = pr * e2.x - pi * e2.y;  // cos(k . x)
                const double2 g01 = kg[q], g23 = kg[kDenseKT + q], g45 = kg[2 * kDenseKT + q];
                s[0] = fma(g01.x, cv, s[0]);
                s[1] = fma(g01.y, cv, s[1]);
                s[2] = fma(g23.x, cv, s[2]);
                s[3] = fma(g23.y, cv, s[3]);
                s[4] = fma(g45.x, cv, s[4]);
                s[5] = fma(g45.y, cv, s[5]);
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 6; q++)
        for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(kFull, s[q], o);
    if (lane == 0 && live) {
        const size_t ld = 3 * (size_t)A.m;
        double blk[3][3] = {{s[0], s[3], s[4]}, {s[3], s[1], s[5]}, {s[4], s[5], s[2]}};
        for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) dA[(3 * (size_t)j + c) * ld + 3 * (size_t)i + r] += blk[r][c];
    }
}

int launch_dense_matrix(double* dA, const double* dx, int m, const double* dx0, int n, double a, double d, double e,
                        const int* Mx, const int* Nx, const double* L, int tau_scaled, cudaStream_t s)
{
    if (m <= 0 || n <= 0) return 0;
    for (int q = 0; q < 3; q++)
        if (Nx[q] > kDenseMaxN) return -4;
    DenseArgs A;
    A.a = a;
    A.d = d;
    A.e = e;
    A.c_d = -expm1(-a * a * d * d / 4);
    A.c_e = -expm1(-a * a * e * e / 4);
    A.tau_inv = tau_scaled ? 1.0 / (L[0] * L[1] * L[2]) : 1.0;
    for (int q = 0; q < 3; q++) {
        A.L[q] = L[q];
        A.Mx[q] = Mx[q] < 0 ? -1 : Mx[q];
        A.Nx[q] = Nx[q] < 0 ? 0 : Nx[q];
    }
    A.m = m;
    A.n = n;
    int tab_len = (2 * A.Nx[0] + 1) + (2 * A.Nx[1] + 1) + (2 * A.Nx[2] + 1);
    size_t smem = (size_t)kDenseKT * (3 * sizeof(double2) + sizeof(int)) + (size_t)kDenseWarps * tab_len * sizeof(double2);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    long long pairs = (long long)m * n;
    unsigned blocks = (unsigned)((pairs + kDenseWarps - 1) / kDenseWarps);
    if (A.Mx[0] < 0 || A.Mx[1] < 0 || A.Mx[2] < 0) A.Mx[0] = A.Mx[1] = A.Mx[2] = -1;
    k_dense<<<blocks, kDenseWarps * 32, smem, s>>>(dA, dx, dx0, A);
    return 0;
}

}  // namespace pb
