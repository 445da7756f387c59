// Plain-old-data types shared by host code and CUDA kernels.
#pragma once
#include <stdint.h>

namespace pb {

// 32-byte aligned 4-vector of doubles (a record of one particle in FP64 mode).
struct alignas(32) Dbl4 {
    double x, y, z, w;
};
#ifdef __CUDACC__
__host__ __device__
#endif
    inline Dbl4
    make_dbl4(double x, double y, double z, double w)
{
    Dbl4 v;
    v.x = x;
    v.y = y;
    v.z = z;
    v.w = w;
    return v;
}

constexpr int kMaxPoly = 28;    // max polynomial terms per real-space table
constexpr int kNumSeries = 16;  // terms of the FP64 small-r series

// Per-instance real-space kernel tables (built in FP64 on the host).
//   r >= r_tiny:  H1 = (Td1(t) - [r<rs] Te1(te)) / r,  H2 = (Td2 - [r<rs] Te2) / r^3
//                 with t = r*td_scale + td_off in [-1,1] over [0, rc] and
//                 te = r*te_scale + te_off over [0, rs]; Td/Te are r*H1, r^3*H2
//                 of S - R_d and S - R_eps (monomial coefficients, FP32).
//   r <  r_tiny:  H = R_eps - R_d from its power series in r^2 (FP64).
struct PbTables {
    float pd1[kMaxPoly], pd2[kMaxPoly];
    float pe1[kMaxPoly], pe2[kMaxPoly];
    int nd, ne;
    float td_scale, td_off, te_scale, te_off;
    float rc2, rs2, rtiny2f;
    int blob;  // eps > 0
    double ser1[kNumSeries], ser2[kNumSeries];
    double self1;   // H1 at r = 0
    double rtiny2;  // r_tiny^2
};

// Per-instance descriptor, resident on the device for multi-instance kernels.
struct PbInst {
    double L[3];
    double alpha, eps, d;
    double rc;
    double h[3];      // cell widths
    double gh[3];     // grid spacings
    double eta;       // Gaussian spreading parameter: exp(-r^2/eta)
    double kfac;      // spectral prefactor (normalisations of spread, FFT, gather)
    double zero_mode[3];  // k = 0 mean-flow velocity added to every target (or 0)
    int nc[3];        // cells per axis
    int S[3];         // stencil reach per axis (cells)
    int M[3];         // FFT grid
    int P;            // Gaussian support (points), max over axes
    int Pa[3];        // Gaussian support per axis
    int n_src, n_tgt;
    int src_off, tgt_off;     // offsets into the packed particle arrays
    int cell_off, ncell;      // offset into the packed cell arrays
    long long grid_off;       // offset (real elements) of the instance's grid (4 values per point:
                              // FP32 interleaved xyz+pad, FP64 three planes + an unused one)
    long long spec_off;       // offset (complex elements) of component 0 of the spectrum
    int flags;
    int same;                 // targets are the sources
    int bucket;               // FFT size bucket
    int pad;
};

}  // namespace pb
