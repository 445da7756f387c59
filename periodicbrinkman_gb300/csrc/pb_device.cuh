// Device-side helpers shared by the CUDA translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pb_types.h"

namespace pb {

constexpr double kPiD = 3.14159265358979323846264338327950288;
constexpr unsigned kFull = 0xffffffffu;

// Error-free sum: s + e == a + b exactly (Knuth).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// Split a double into a float pair hi + lo.
__host__ __device__ __forceinline__ void split_double(double x, float& hi, float& lo)
{
    hi = (float)x;
    lo = (float)(x - (double)hi);
}

// Kahan-compensated accumulation: the running sum is s - c.
__device__ __forceinline__ void kahan_add(float& s, float& c, float v)
{
    float y = v - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
}

__device__ __forceinline__ double wrap_coord(double v, double L)
{
    double w = v - L * floor(v / L);
    if (w >= L) w -= L;
    if (w < 0) w = 0;
    return w;
}

// As wrap_coord with the inverse length given (no FP64 division; the
// rounding of v * iL is absorbed by the range fix-up).
__device__ __forceinline__ double wrap_coord_r(double v, double L, double iL)
{
    double w = fma(-L, floor(v * iL), v);
    if (w >= L) w -= L;
    if (w < 0) w = 0;
    return w;
}

__device__ __forceinline__ int find_instance(const int* offsets, int ninst, int idx)
{
    // offsets: ninst+1 ascending prefix; returns q with offsets[q] <= idx < offsets[q+1]
    int lo = 0, hi = ninst - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (offsets[mid] <= idx)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Closed-form diffH of the reference in FP64 (cuda/periodicBrinkman.h:85-112), r > 0.
__device__ __forceinline__ double experf_d(double x, double z)
{
    return ((x * z < 0) || (x * x + z * z < 700)) ? exp(2 * x * z) * erfc(z + x) : 0.0;
}

__device__ __forceinline__ void diffH_d(double r, double a, double d, double c_d, double& H1, double& H2)
{
    // c_d = 1 - exp(-a^2 d^2 / 4)
    const double kSqrtPi = 1.77245385090551602729816748334114518;
    double r2 = r * r;
    double ex = exp(-r2 / (d * d)) * c_d;
    double ec = erfc(r / d);
    double em = experf_d(-a * d / 2, r / d), ep = experf_d(a * d / 2, r / d);
    double pre = 1.0 / (8 * kPiD * a * a * r2 * r);
    double g = 1.0 / (2 * a * a * d * d * d * kPiD * kSqrtPi);
    double ar = a * r, a2r2 = a * a * r2;
    H1 = -2 * pre * ec - (d * d + 2 * r2) * g / r2 * ex + pre * ((1 + ar + a2r2) * em + (1 - ar + a2r2) * ep);
    H2 = 6 * pre / r2 * ec + (3 * d * d + 2 * r2) * g / (r2 * r2) * ex -
         pre / r2 * ((3 + 3 * ar + a2r2) * em + (3 - 3 * ar + a2r2) * ep);
}

// diffH_d with the per-(alpha, delta) constants hoisted and one division per
// call (1/r) instead of eight: the FP64 pipe of a GB300 runs at a small
// fraction of its FP32 rate and a division is a sequence of FP64 FMAs.  The
// same closed forms (the reference's diffH), rounded differently.
struct DiffHConsts {
    double a, a2, d2, inv_d, inv_d2, c_d, g, inv8pia2, ad2;
};

__device__ __forceinline__ DiffHConsts diffh_consts(double a, double d, double c_d)
{
    const double kSqrtPi = 1.77245385090551602729816748334114518;
    DiffHConsts k;
    k.a = a;
    k.a2 = a * a;
    k.d2 = d * d;
    k.inv_d = 1.0 / d;
    k.inv_d2 = k.inv_d * k.inv_d;
    k.c_d = c_d;
    k.g = 1.0 / (2 * a * a * d * d * d * kPiD * kSqrtPi);
    k.inv8pia2 = 1.0 / (8 * kPiD * a * a);
    k.ad2 = a * d / 2;
    return k;
}

__device__ __forceinline__ void diffH_fast_d(double r, double ir, const DiffHConsts& k, double& H1, double& H2)
{
    const double r2 = r * r, ir2 = ir * ir, z = r * k.inv_d;
    const double ex = exp(-r2 * k.inv_d2) * k.c_d;
    const double ec = erfc(z);
    const double em = experf_d(-k.ad2, z), ep = experf_d(k.ad2, z);
    const double pre = k.inv8pia2 * ir2 * ir;
    const double ar = k.a * r, a2r2 = k.a2 * r2;
    const double gx = k.g * ir2 * ex;
    H1 = -2 * pre * ec - (k.d2 + 2 * r2) * gx + pre * ((1 + ar + a2r2) * em + (1 - ar + a2r2) * ep);
    H2 = 6 * pre * ir2 * ec + (3 * k.d2 + 2 * r2) * gx * ir2 -
         pre * ir2 * ((3 + 3 * ar + a2r2) * em + (3 - 3 * ar + a2r2) * ep);
}

// FP64 small-r series of R_eps - R_d in r^2.
__device__ __forceinline__ void series_H(const PbTables& T, double r2, double& H1, double& H2)
{
    double s1 = T.ser1[kNumSeries - 1], s2 = T.ser2[kNumSeries - 1];
#pragma unroll
    for (int m = kNumSeries - 2; m >= 0; m--) {
        s1 = fma(s1, r2, T.ser1[m]);
        s2 = fma(s2, r2, T.ser2[m]);
    }
    H1 = s1;
    H2 = s2;
}

}  // namespace pb
