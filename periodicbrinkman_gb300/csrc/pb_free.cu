// Free-space (non-periodic) Brinkmanlet on the GPU: the regularized
// Brinkmanlet R_eps (eps > 0) or the singular one S (eps = 0) of the
// reference's Brinkmanlet() (cuda/periodicBrinkman.h:119-141, with regH
// 53-78 and singH 31-46), as a direct FP64 sum of velocities
// u(y_i) = sum_j (H1 I + H2 x x^T) f_j, x = y_i - x_j, or as the dense
// 3m x 3n matrix of those tensors.
//
// Evaluation (FP64), chosen so that no form cancels:
//   eps > 0, r < eps/2 : the power series of R_eps in r^2 (built on the host
//                        from the radial Fourier integral of the blob);
//   eps > 0, otherwise : the reference's closed forms of regH;
//   eps = 0            : S as A1(u)/(4 pi r), A2(u)/(4 pi r^3), u = alpha r,
//                        with A1, A2 from their power series below u = 1/2
//                        (the closed forms lose (alpha r)^-2 of relative
//                        precision there) and from the closed forms above.
// With eps = 0 a coincident pair (r below 1e-12, the reference's switch
// radius) has no finite velocity: the velocity sum skips it, and the matrix
// carries the reference's sentinel 1.79e308 on its diagonal as singH does.
// The sums are O(m n): this is the free-space companion of the periodic
// solver for small problems, not a fast method.
#include <cmath>
#include <cstring>
#include <vector>

#include "pb_device.cuh"
#include "pb_internal.h"
#include "pb_kernel_math.h"
#include "pbrinkman.h"

namespace pb {
namespace {

constexpr int kFreeSer = 28;  // terms of the R_eps series in r^2
constexpr int kSingSer = 24;  // terms of the A1, A2 series in u
constexpr int kFreeBlock = 128;
constexpr double kSwitch = 1e-12;  // the reference's switch radius (its eps)

struct FreeArgs {
    double a, eps, rser2;                  // rser2 = (eps/2)^2: the series below it
    double ser1[kFreeSer], ser2[kFreeSer];  // R_eps: H1 = sum ser1[m] r^2m, H2 = sum ser2[m] r^2m
    double s1[kSingSer], s2[kSingSer];      // A1 = sum s1[k] u^k, A2 = sum s2[k] u^k
};

__device__ __forceinline__ void free_H(const FreeArgs& A, double r2, double& H1, double& H2)
{
    const double kSqrtPi = 1.77245385090551602729816748334114518;
    const double a = A.a;
    if (A.eps > 0) {
        if (r2 < A.rser2) {
            double h1 = A.ser1[kFreeSer - 1], h2 = A.ser2[kFreeSer - 1];
#pragma unroll
            for (int m = kFreeSer - 2; m >= 0; m--) {
                h1 = fma(h1, r2, A.ser1[m]);
                h2 = fma(h2, r2, A.ser2[m]);
            }
            H1 = h1;
            H2 = h2;
            return;
        }
        const double d = A.eps, r = sqrt(r2), ir = 1.0 / r, ir2 = ir * ir;
        const double expx2 = exp(-r2 / (d * d)), Erf = erf(r / d), c = -expm1(-a * a * d * d / 4);
        const double pre = ir2 * ir / (8 * kPiD * a * a);
        const double g = c * expx2 / (2 * a * a * d * d * d * kPiD * kSqrtPi);
        const double em = experf_d(a * d / 2, -r / d), ep = experf_d(a * d / 2, r / d);
        const double ar = a * r, a2r2 = a * a * r2;
        H1 = -2 * pre * Erf + g * (d * d + 2 * r2) * ir2 + pre * ((1 + ar + a2r2) * em - (1 - ar + a2r2) * ep);
        H2 = 6 * pre * ir2 * Erf - g * (3 * d * d + 2 * r2) * ir2 * ir2 -
             pre * ir2 * ((3 + 3 * ar + a2r2) * em - (3 - 3 * ar + a2r2) * ep);
        return;
    }
    const double r = sqrt(r2), u = a * r;
    double A1, A2;
    if (u < 0.5) {
        A1 = A.s1[kSingSer - 1];
        A2 = A.s2[kSingSer - 1];
#pragma unroll
        for (int k = kSingSer - 2; k >= 0; k--) {
            A1 = fma(A1, u, A.s1[k]);
            A2 = fma(A2, u, A.s2[k]);
        }
    } else {
        const double em = exp(-u), iu2 = 1.0 / (u * u);
        A1 = (-1 + em * (1 + u + u * u)) * iu2;
        A2 = (3 - em * (3 + 3 * u + u * u)) * iu2;
    }
    H1 = A1 / (4 * kPiD * r);
    H2 = A2 / (4 * kPiD * r * r2);
}

// One thread per target; sources staged through shared memory a block at a time.
__global__ void __launch_bounds__(kFreeBlock)
    k_free_velocity(const double* __restrict__ y, int m, const double* __restrict__ x, const double* __restrict__ f,
                    int n, const FreeArgs A, double* __restrict__ U)
{
    __shared__ double sx[3][kFreeBlock], sf[3][kFreeBlock];
    const int i = blockIdx.x * kFreeBlock + threadIdx.x;
    double yi[3] = {0, 0, 0};
    if (i < m)
        for (int c = 0; c < 3; c++) yi[c] = y[3 * (size_t)i + c];
    double u0 = 0, u1 = 0, u2 = 0;
    const double sw2 = kSwitch * kSwitch;
    for (int base = 0; base < n; base += kFreeBlock) {
        const int j = base + threadIdx.x;
        if (j < n)
            for (int c = 0; c < 3; c++) {
                sx[c][threadIdx.x] = x[3 * (size_t)j + c];
                sf[c][threadIdx.x] = f[3 * (size_t)j + c];
            }
        __syncthreads();
        const int cnt = min(kFreeBlock, n - base);
        if (i < m)
            for (int k = 0; k < cnt; k++) {
                const double dx = yi[0] - sx[0][k], dy = yi[1] - sx[1][k], dz = yi[2] - sx[2][k];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (A.eps == 0 && r2 <= sw2) continue;  // coincident singular pair: no finite velocity
                double H1, H2;
                free_H(A, r2, H1, H2);
                const double fx = sf[0][k], fy = sf[1][k], fz = sf[2][k];
                const double g = H2 * (fx * dx + fy * dy + fz * dz);
                u0 += H1 * fx + g * dx;
                u1 += H1 * fy + g * dy;
                u2 += H1 * fz + g * dz;
            }
        __syncthreads();
    }
    if (i < m) {
        U[3 * (size_t)i] = u0;
        U[3 * (size_t)i + 1] = u1;
        U[3 * (size_t)i + 2] = u2;
    }
}

// One thread per (target i, source j): dA(3i + r, 3j + c) += H1 delta_rc + H2 x_r x_c.
__global__ void k_free_matrix(double* __restrict__ dA, const double* __restrict__ dx, int m,
                              const double* __restrict__ dx0, int n, const FreeArgs A)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)m * n) return;
    const int i = (int)(t % m), j = (int)(t / m);
    double xh[3];
    for (int c = 0; c < 3; c++) xh[c] = dx[3 * (size_t)i + c] - dx0[3 * (size_t)j + c];
    const double r2 = xh[0] * xh[0] + xh[1] * xh[1] + xh[2] * xh[2];
    double H1, H2;
    if (A.eps == 0 && r2 <= kSwitch * kSwitch) {
        H1 = H2 = 1.79e+308;  // singH's sentinel (cuda/periodicBrinkman.h:44)
    } else {
        free_H(A, r2, H1, H2);
    }
    const size_t ld = 3 * (size_t)m;
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) {
            double v = xh[r] * xh[c] * H2;
            if (r == c) v += H1;
            dA[(3 * (size_t)j + c) * ld + 3 * (size_t)i + r] += v;
        }
}

int free_args(double alpha, double eps, FreeArgs& A)
{
    if (!std::isfinite(alpha) || !(alpha > 0) || !std::isfinite(eps) || eps < 0)
        return api_error(PB_ERR_INVALID, "need alpha > 0 and eps >= 0");
    std::memset(&A, 0, sizeof(A));
    A.a = alpha;
    A.eps = eps;
    A.rser2 = 0.25 * eps * eps;
    if (eps > 0) regularized_series(alpha, eps, kFreeSer, A.ser1, A.ser2);
    // A1 = sum_{k>=2} (-1)^k (k-1)^2/k! u^{k-2}, A2 = -sum_{k>=2} (-1)^k (k-1)(k-3)/k! u^{k-2}:
    // the Taylor series of the closed forms (-1 + e^{-u}(1+u+u^2))/u^2 and (3 - e^{-u}(3+3u+u^2))/u^2
    double fact = 2;  // k!
    for (int k = 2; k < kSingSer + 2; k++) {
        const double sg = (k & 1) ? -1.0 : 1.0;
        A.s1[k - 2] = sg * (k - 1.0) * (k - 1.0) / fact;
        A.s2[k - 2] = -sg * (k - 1.0) * (k - 3.0) / fact;
        fact *= (k + 1);
    }
    return PB_OK;
}

}  // namespace
}  // namespace pb

using namespace pb;

extern "C" int pb_brinkmanlet(double* U, const double* y, int m, const double* x, const double* f, int n,
                              double alpha, double eps, int where, void* stream)
{
    NvtxRange nv("pb_brinkmanlet");
    if (m < 0 || n < 0) return api_error(PB_ERR_INVALID, "negative count");
    if (where != PB_HOST && where != PB_DEVICE) return api_error(PB_ERR_INVALID, "bad memory location");
    FreeArgs A;
    int rc = free_args(alpha, eps, A);
    if (rc) return rc;
    if (m == 0) return PB_OK;
    if (!U || !y || (n > 0 && (!x || !f))) return api_error(PB_ERR_INVALID, "null buffer");
    if (pb_device_count() <= 0) return api_error(PB_ERR_CUDA, "no CUDA device");
    cudaStream_t s = (cudaStream_t)stream;
    if (where == PB_DEVICE) {
        k_free_velocity<<<(m + kFreeBlock - 1) / kFreeBlock, kFreeBlock, 0, s>>>(y, m, x, f, n, A, U);
        cudaError_t e = cudaGetLastError();
        return e == cudaSuccess ? PB_OK : api_error(PB_ERR_CUDA, cudaGetErrorString(e));
    }
    for (size_t k = 0; k < 3 * (size_t)m; k++)
        if (!std::isfinite(y[k])) return api_error(PB_ERR_INVALID, "non-finite target");
    for (size_t k = 0; k < 3 * (size_t)n; k++)
        if (!std::isfinite(x[k]) || !std::isfinite(f[k])) return api_error(PB_ERR_INVALID, "non-finite input");
    const size_t bm = 3 * (size_t)m * sizeof(double), bn = 3 * (size_t)std::max(n, 1) * sizeof(double);
    char* buf = nullptr;
    if (cudaMalloc(&buf, 2 * bm + 2 * bn) != cudaSuccess) {
        cudaGetLastError();
        return api_error(PB_ERR_NOMEM, "device allocation failed");
    }
    double *dy = (double*)buf, *dU = (double*)(buf + bm), *dx = (double*)(buf + 2 * bm), *df = (double*)(buf + 2 * bm + bn);
    cudaError_t e = cudaMemcpyAsync(dy, y, bm, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n > 0) e = cudaMemcpyAsync(dx, x, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && n > 0) e = cudaMemcpyAsync(df, f, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        k_free_velocity<<<(m + kFreeBlock - 1) / kFreeBlock, kFreeBlock, 0, s>>>(dy, m, dx, df, n, A, dU);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(U, dU, bm, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(buf);
    return e == cudaSuccess ? PB_OK : api_error(PB_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" int pb_brinkmanlet_matrix(double* dA, const double* dx, int m, const double* dx0, int n, double alpha,
                                     double eps, void* stream)
{
    NvtxRange nv("pb_brinkmanlet_matrix");
    if (m < 0 || n < 0) return api_error(PB_ERR_INVALID, "negative count");
    FreeArgs A;
    int rc = free_args(alpha, eps, A);
    if (rc) return rc;
    if (m == 0 || n == 0) return PB_OK;
    if (!dA || !dx || !dx0) return api_error(PB_ERR_INVALID, "null buffer");
    if (pb_device_count() <= 0) return api_error(PB_ERR_CUDA, "no CUDA device");
    const long long total = (long long)m * n;
    k_free_matrix<<<(unsigned)((total + 255) / 256), 256, 0, (cudaStream_t)stream>>>(dA, dx, m, dx0, n, A);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PB_OK : api_error(PB_ERR_CUDA, cudaGetErrorString(e));
}
