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

constexpr int kMaxPoly = 28;    // max terms of the far polynomial (held in registers)
constexpr int kMaxCheb = 40;    // max terms of the near and blob Chebyshev series (shared memory)
constexpr int kNumSeries = 16;  // terms of the FP64 small-r series
constexpr int kMaxCheb64 = 48;  // max terms of the FP64 far Chebyshev series (FP64 path)
constexpr int kItemCells = 32;  // bound of the cells along z of a real-space work item (PbInst::zspan)
constexpr int kCapItems = 1;    // execution status bit: real-space work items beyond the item array
constexpr int kScanStall = 2;   // execution status bit: a cell-count scan gave up waiting for a predecessor

// Per-instance real-space kernel tables (built in FP64 on the host).  The pair
// kernel H = (R_eps - R_d) inside the blob region, S - R_d outside it, is
// evaluated in FP32 by pieces chosen so that no piece cancels:
//   far   r in [r_mid, rc]: T1 = r*H1, T2 = r^3*H2 of S - R_d, monomial
//         coefficients in t = r*td_scale + td_off in [-1, 1] (Horner, registers)
//   near  r in [rs, r_mid]: the same T of S - R_d as a Chebyshev series in
//         t = r*tn_scale + tn_off (Clenshaw)
//   blob  r in [0, rs] (eps > 0): H1 and r^2*H2 of R_eps - R_d as a Chebyshev
//         series in t = r*tb_scale + tb_off (Clenshaw)
//   r < r_tiny (eps > 0): H = R_eps - R_d from its FP64 power series in r^2.
// Most pairs lie in the far piece; the other pieces are the rare path.
struct PbTables {
    float pd1[kMaxPoly], pd2[kMaxPoly];  // far piece (monomial)
    float cn1[kMaxCheb], cn2[kMaxCheb];  // near piece (Chebyshev)
    float cb1[kMaxCheb], cb2[kMaxCheb];  // blob piece (Chebyshev)
    int nd, nn, nb;
    float td_scale, td_off, tn_scale, tn_off, tb_scale, tb_off;
    float rc2, rm2, rs2, rtiny2f;
    int blob;  // eps > 0
    double ser1[kNumSeries], ser2[kNumSeries];
    double self1;   // H1 at r = 0
    double rtiny2;  // r_tiny^2
    // FP64 path: the far piece (T1, T2 of S - R_d for r in [r_mid, rc]) as an
    // FP64 Chebyshev series in t = r*tf_scale + tf_off (Clenshaw), fitted to
    // 1e-14 of its largest coefficient; pairs below r_mid use the closed forms
    double cf1[kMaxCheb64], cf2[kMaxCheb64];
    double tf_scale, tf_off, rf2;  // argument map; r_mid^2
    int nf;
};

// Per-instance descriptor, resident on the device for multi-instance kernels.
struct PbInst {
    double L[3];
    double alpha, eps, d;
    double rc;
    double h[3];      // cell widths
    double gh[3];     // grid spacings
    double gih[3];    // inverse grid spacings (M / L)
    double iL[3];     // inverse box lengths
    double ih[3];     // inverse cell widths
    double eta;       // Gaussian spreading parameter: exp(-r^2/eta)
    float ghh[3], ghl[3];  // grid spacings as FP32 hi + lo (window set-up without FP64)
    float gihf[3];         // inverse grid spacings in FP32
    float inv_eta_f;       // 1 / eta in FP32
    float hch[3], hcl[3];  // cell widths as FP32 hi + lo (real-space frames without FP64)
    float Lh[3], Ll[3];    // box lengths as FP32 hi + lo
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
    int csplit;               // real-space work items per row item (stencil columns split into groups)
    int zspan;                // max cells along z of a real-space work item (<= kItemCells)
};

}  // namespace pb
