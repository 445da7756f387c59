// k-space Ewald sum by spectral Ewald: Gaussian spreading of the three force
// components onto an M^3 grid, batched 3D real FFT, multiplication by the
// screened Brinkman Green tensor with Gaussian deconvolution, inverse FFT and
// Gaussian gather (the algorithm of cuda/fftBrinkman.h:101-273, with a
// centred support window, no spectrum conjugation and per-target support
// gather).  Also the final FP64 combine of real space, k space, self and the
// optional k = 0 mode.
//
// FFT: hand-written passes along z (real-to-complex by the packed half-length
// transform), y, and x: register-resident four-step line transforms for FP32
// grids with lines of 4 to 256 points, shared-memory Stockham radix-2 passes
// for FP64 grids and longer lines.  The x pass of the forward transform is
// fused with the Green multiplication and the x pass of the inverse, so the
// spectrum is read and written once for all three.
#include <algorithm>

#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

template <class T>
struct Cx;
template <>
struct Cx<float> {
    typedef float2 t;
};
template <>
struct Cx<double> {
    typedef double2 t;
};

template <class T2>
__device__ __forceinline__ T2 cmul(T2 a, T2 b)
{
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// ---------------------------------------------------------------------------
// Spreading and gathering
// ---------------------------------------------------------------------------

// Sorted positions: mixed (float4 hi, float4 lo, instance in hi.w bits) or FP64 (Dbl4, instance in w).
__device__ __forceinline__ void load_pos(const float4* a, const float4* b, int i, double* x, int& q)
{
    float4 h = a[i], l = b[i];
    x[0] = (double)h.x + (double)l.x;
    x[1] = (double)h.y + (double)l.y;
    x[2] = (double)h.z + (double)l.z;
    q = __float_as_int(h.w);
}
__device__ __forceinline__ void load_pos(const Dbl4* a, const Dbl4* /*b*/, int i, double* x, int& q)
{
    Dbl4 h = a[i];
    x[0] = h.x;
    x[1] = h.y;
    x[2] = h.z;
    q = (int)h.w;
}
__device__ __forceinline__ void load_frc(const float4* f, int i, double* v)
{
    float4 h = f[i];
    v[0] = h.x;
    v[1] = h.y;
    v[2] = h.z;
}
__device__ __forceinline__ void load_frc(const Dbl4* f, int i, double* v)
{
    Dbl4 h = f[i];
    v[0] = h.x;
    v[1] = h.y;
    v[2] = h.z;
}

constexpr int kSpreadWarps = 8;
constexpr int kMaxP = 32;

// Spreading visits the cell-sorted points in an interleaved order (64 strands
// through the sorted array), so warps in flight at the same time work on points
// far apart and their atomics spread over the grid instead of piling onto the
// same cache lines.  Returns -1 past the end.
__device__ __forceinline__ int spread_order(int s, int ntot)
{
    const int R = (ntot + 63) >> 6;
    const int p = (s & 63) * R + (s >> 6);
    return (s < 64 * R && p < ntot) ? p : -1;
}

// Lanes own positions of the y-z plane of the window (and, for windows with
// fewer than 32 y-z points, a residue class of x) and loop over x, so the
// inner loops carry no index division.  `xs` = first x of the lane, `R` = x step.
__device__ __forceinline__ int window_lanes(int Py, int Pz) { return Py * Pz >= 32 ? 1 : 32 / (Py * Pz); }

// Per-axis Gaussian weights exp(-(x - (g0+p) h)^2 / eta) and wrapped grid
// indices of the P-point window centred on x (lane p computes entry p).
template <class T>
__device__ __forceinline__ void window(const PbInst& I, const double* x, int lane, T (*wgt)[kMaxP],
                                       int (*idx)[kMaxP])
{
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int P = I.Pa[a];
        if (lane < P) {
            double h = I.gh[a];
            int g0 = (int)floor(x[a] / h) - P / 2 + 1;
            double base = x[a] - (double)g0 * h;
            T dx = (T)(base - (double)lane * h);
            wgt[a][lane] = exp(-dx * dx / (T)I.eta);
            int g = (g0 + lane) % I.M[a];
            idx[a][lane] = g < 0 ? g + I.M[a] : g;
        }
    }
}

template <class T, class PV, class FV>
__global__ void __launch_bounds__(kSpreadWarps * 32)
    k_spread(const PbInst* __restrict__ inst, const int* __restrict__ ntot_p, const PV* __restrict__ pa,
             const PV* __restrict__ pb, const FV* __restrict__ frc, T* __restrict__ grid)
{
    const int ntot = *ntot_p;
    __shared__ T wgt[kSpreadWarps][3][kMaxP];
    __shared__ int gidx[kSpreadWarps][3][kMaxP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = spread_order(blockIdx.x * kSpreadWarps + w, ntot);
    if (s < 0) return;
    double x[3], fv[3];
    int q;
    load_pos(pa, pb, s, x, q);
    load_frc(frc, s, fv);
    const PbInst& I = inst[q];
    window<T>(I, x, lane, wgt[w], gidx[w]);
    __syncwarp();
    const int Px = I.Pa[0], Py = I.Pa[1], Pz = I.Pa[2], P2 = Py * Pz, R = window_lanes(Py, Pz);
    const size_t comp = (size_t)I.M[0] * I.M[1] * I.M[2], M12 = (size_t)I.M[1] * I.M[2];
    T* g0 = grid + I.grid_off;
    for (int id = lane; id < P2 * R; id += 32) {
        const int xs = id / P2, yz = id - xs * P2, py = yz / Pz, pz = yz - py * Pz;
        const T wyz = wgt[w][1][py] * wgt[w][2][pz];
        const T h0 = (T)fv[0] * wyz, h1 = (T)fv[1] * wyz, h2 = (T)fv[2] * wyz;
        const size_t oyz = (size_t)gidx[w][1][py] * I.M[2] + gidx[w][2][pz];
        for (int px = xs; px < Px; px += R) {
            const T wx = wgt[w][0][px];
            const size_t o = (size_t)gidx[w][0][px] * M12 + oyz;
            atomicAdd(g0 + o, h0 * wx);
            atomicAdd(g0 + comp + o, h1 * wx);
            atomicAdd(g0 + 2 * comp + o, h2 * wx);
        }
    }
}

template <class T, class PV>
__global__ void __launch_bounds__(kSpreadWarps * 32)
    k_gather(const PbInst* __restrict__ inst, const int* __restrict__ ntot_p, const PV* __restrict__ pa,
             const PV* __restrict__ pb, const T* __restrict__ grid, T* __restrict__ u_k)
{
    const int ntot = *ntot_p;
    __shared__ T wgt[kSpreadWarps][3][kMaxP];
    __shared__ int gidx[kSpreadWarps][3][kMaxP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int s = blockIdx.x * kSpreadWarps + w;
    if (s >= ntot) return;
    double x[3];
    int q;
    load_pos(pa, pb, s, x, q);
    const PbInst& I = inst[q];
    window<T>(I, x, lane, wgt[w], gidx[w]);
    __syncwarp();
    const int Px = I.Pa[0], Py = I.Pa[1], Pz = I.Pa[2], P2 = Py * Pz, R = window_lanes(Py, Pz);
    const size_t comp = (size_t)I.M[0] * I.M[1] * I.M[2], M12 = (size_t)I.M[1] * I.M[2];
    const T* g0 = grid + I.grid_off;
    // plain FP64 sums (x rows by FMA, then weighted by the row's y-z weight):
    // a few hundred same-sign-weighted terms per lane lose ~1e-14, and GB300's
    // FP64 pipe is the limit here (compensated sums per point cost 4x the work)
    T s0 = 0, s1 = 0, s2 = 0;
    for (int id = lane; id < P2 * R; id += 32) {
        const int xs = id / P2, yz = id - xs * P2, py = yz / Pz, pz = yz - py * Pz;
        const T wyz = wgt[w][1][py] * wgt[w][2][pz];
        const size_t oyz = (size_t)gidx[w][1][py] * I.M[2] + gidx[w][2][pz];
        T r0 = 0, r1 = 0, r2 = 0;
        for (int px = xs; px < Px; px += R) {
            const T wx = wgt[w][0][px];
            const size_t o = (size_t)gidx[w][0][px] * M12 + oyz;
            r0 = fma(wx, __ldg(g0 + o), r0);
            r1 = fma(wx, __ldg(g0 + comp + o), r1);
            r2 = fma(wx, __ldg(g0 + 2 * comp + o), r2);
        }
        s0 = fma(wyz, r0, s0);
        s1 = fma(wyz, r1, s1);
        s2 = fma(wyz, r2, s2);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(kFull, s0, o);
        s1 += __shfl_xor_sync(kFull, s1, o);
        s2 += __shfl_xor_sync(kFull, s2, o);
    }
    if (lane == 0) {
        u_k[3 * (size_t)s] = s0;
        u_k[3 * (size_t)s + 1] = s1;
        u_k[3 * (size_t)s + 2] = s2;
    }
}

// FP32 grids interleave the three components of a point in one float4, so a
// point costs one vector atomic (spread) or one 16-byte load (gather).
// FP32-grid window of a point given as FP32 hi/lo pairs: lane a < 3 resolves
// axis a (the grid cell holding x, by a multiply with the inverse spacing, and
// the offset of x from the window start in double-float arithmetic: g0 h is
// split exactly by an FMA), the other lanes take those by shuffle, and lane
// p < P computes weight p from the offset.  No FP64: the FP64 pipe of this GPU
// runs at a small fraction of the FP32 rate, and the FP64 window set-up had
// kept it 35-40% busy in spreading and gathering.  Near a cell boundary the
// cell may come out one lower or higher than exact arithmetic would give; the
// window then still holds the point within half a spacing of its centre.
__device__ __forceinline__ void window_f32(const PbInst& I, float4 h4, float4 l4, int lane, float (*wgt)[kMaxP],
                                           int (*idx)[kMaxP], int* g0out = nullptr)
{
    int g0 = 0;
    float base = 0.f;
    if (lane < 3) {
        const float xh = lane == 0 ? h4.x : lane == 1 ? h4.y : h4.z;
        const float xl = lane == 0 ? l4.x : lane == 1 ? l4.y : l4.z;
        const float gi = I.gihf[lane];
        const int c = min(max((int)floorf(fmaf(xh, gi, xl * gi)), 0), I.M[lane] - 1);
        g0 = c - I.Pa[lane] / 2 + 1;
        const float gf = (float)g0, hh = I.ghh[lane];
        const float p = gf * hh, e = fmaf(gf, hh, -p);  // g0 hh = p + e exactly
        base = ((xh - p) - e) + (xl - gf * I.ghl[lane]);
        if (g0out) g0out[lane] = g0;
    }
    const float inv_eta = I.inv_eta_f;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int ga = __shfl_sync(kFull, g0, a);
        const float ba = __shfl_sync(kFull, base, a);
        if (lane < I.Pa[a]) {
            const float dx = fmaf(-(float)lane, I.ghh[a], ba);
            wgt[a][lane] = expf(-dx * dx * inv_eta);
            idx[a][lane] = (ga + lane) & (I.M[a] - 1);  // grids are powers of two
        }
    }
}

// Grouped spreading: a warp takes kSpreadGroup consecutive (cell-sorted, so
// nearby) points and adds their windows together over the box that holds
// them all, one vector L2 atomic per box point instead of one per point and
// window point (about half the atomics for four points of one cell).  Each box
// point sums the points' contributions in registers; per-point weights are
// laid out along the box (zero outside the point's window), so the box loops
// need no bounds tests.  Points of another instance, or a box wider than
// kBoxMax along an axis, are spread one point at a time through the same loops.
constexpr int kSpreadGroup = 4;  // measured at N = 1e5: 2 -> 0.31 ms, 3 -> 0.26, 4 -> 0.24, 5 -> 0.244, 6 -> 0.276
constexpr int kBoxMax = 48;

// 4 blocks per SM (64 registers, a few spilled): measured 0.286 ms vs 0.300 at
// 3 blocks (80 registers) and 0.294 / 0.332 at 5 / 6 blocks (N = 1e5)
__global__ void __launch_bounds__(kSpreadWarps * 32, 4)
    k_spread_f4g(const PbInst* __restrict__ inst, const int* __restrict__ ntot_p, const float4* __restrict__ pa,
                 const float4* __restrict__ pb, const float4* __restrict__ frc, float* __restrict__ grid)
{
    constexpr int G = kSpreadGroup;
    __shared__ float wgt[kSpreadWarps][3][kMaxP];
    __shared__ int gidx[kSpreadWarps][3][kMaxP];
    __shared__ float raw[kSpreadWarps][G][3][kMaxP];
    __shared__ float pw[kSpreadWarps][G][3][kBoxMax];
    __shared__ int gs[kSpreadWarps][G][3];
    __shared__ float4 fs[kSpreadWarps][G];
    const int ntot = *ntot_p;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ngroups = (ntot + G - 1) / G;
    const int gi = spread_order(blockIdx.x * kSpreadWarps + w, ngroups);
    if (gi < 0) return;
    const int sb = gi * G, cnt = min(G, ntot - sb);
    const int q0 = __float_as_int(pa[sb].w);
    const PbInst& I = inst[q0];
    bool same = true;
    for (int p = 0; p < cnt; p++) {
        const float4 h4 = pa[sb + p], l4 = pb[sb + p];
        if (__float_as_int(h4.w) != q0) {
            same = false;
            continue;
        }
        window_f32(I, h4, l4, lane, wgt[w], gidx[w], gs[w][p]);
        __syncwarp();
        for (int i = lane; i < 3 * kMaxP; i += 32) raw[w][p][i / kMaxP][i % kMaxP] = wgt[w][i / kMaxP][i % kMaxP];
        if (lane == 0) fs[w][p] = frc[sb + p];
        __syncwarp();
    }
    const int Pa[3] = {I.Pa[0], I.Pa[1], I.Pa[2]};
    int b0[3], B[3];
    bool fits = same;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int lo = 1 << 30, hi = -(1 << 30);
        for (int p = 0; p < cnt; p++) {
            lo = min(lo, gs[w][p][a]);
            hi = max(hi, gs[w][p][a] + Pa[a]);
        }
        b0[a] = lo;
        B[a] = hi - lo;
        fits = fits && B[a] <= kBoxMax;
    }
    const size_t M12 = (size_t)I.M[1] * I.M[2];
    const int mx = I.M[0] - 1, my = I.M[1] - 1, mz = I.M[2] - 1;
    float4* g4 = reinterpret_cast<float4*>(grid + I.grid_off);
    // boxes: the whole group when it fits, else each point of instance q0 alone
    // (points of another instance go through the one-point kernel's path below)
    const int nbox = fits ? 1 : cnt;
    for (int bi = 0; bi < nbox; bi++) {
        int p0 = 0, p1 = cnt;
        int o[3] = {b0[0], b0[1], b0[2]}, L[3] = {B[0], B[1], B[2]};
        if (!fits) {
            p0 = bi;
            p1 = bi + 1;
            if (__float_as_int(pa[sb + bi].w) != q0) continue;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                o[a] = gs[w][bi][a];
                L[a] = Pa[a];
            }
        }
        __syncwarp();
        for (int i = lane; i < G * 3 * kBoxMax; i += 32) {
            const int p = i / (3 * kBoxMax), r = i - p * 3 * kBoxMax, a = r / kBoxMax, x = r - a * kBoxMax;
            float v = 0.f;
            if (p >= p0 && p < p1) {
                const int k = o[a] + x - gs[w][p][a];
                if (x < L[a] && k >= 0 && k < Pa[a]) v = raw[w][p][a][k];
            }
            pw[w][p][a][x] = v;
        }
        __syncwarp();
        float fx[G], fy[G], fz[G];
#pragma unroll
        for (int p = 0; p < G; p++) {
            const float4 f = fs[w][p];
            const bool in = p >= p0 && p < p1;
            fx[p] = in ? f.x : 0.f;
            fy[p] = in ? f.y : 0.f;
            fz[p] = in ? f.z : 0.f;
        }
        const int Byz = L[1] * L[2];
        for (int yz = lane; yz < Byz; yz += 32) {
            const int y = yz / L[2], z = yz - y * L[2];
            float c0[G], c1[G], c2[G];
            bool any = false;
#pragma unroll
            for (int p = 0; p < G; p++) {
                const float wyz = pw[w][p][1][y] * pw[w][p][2][z];
                any = any || wyz != 0.f;
                c0[p] = fx[p] * wyz;
                c1[p] = fy[p] * wyz;
                c2[p] = fz[p] * wyz;
            }
            if (!any) continue;
            const size_t oyz = (size_t)((o[1] + y) & my) * I.M[2] + ((o[2] + z) & mz);
            for (int x = 0; x < L[0]; x++) {
                float v0 = 0.f, v1 = 0.f, v2 = 0.f;
#pragma unroll
                for (int p = 0; p < G; p++) {
                    const float wx = pw[w][p][0][x];
                    v0 = fmaf(c0[p], wx, v0);
                    v1 = fmaf(c1[p], wx, v1);
                    v2 = fmaf(c2[p], wx, v2);
                }
                if (v0 != 0.f || v1 != 0.f || v2 != 0.f)
                    atomicAdd(g4 + (size_t)((o[0] + x) & mx) * M12 + oyz, make_float4(v0, v1, v2, 0.f));
            }
        }
    }
    if (same) return;
    // points of other instances than the group's first: one at a time
    for (int p = 1; p < cnt; p++) {
        const float4 h4 = pa[sb + p], l4 = pb[sb + p], fv = frc[sb + p];
        const int qp = __float_as_int(h4.w);
        if (qp == q0) continue;
        const PbInst& J = inst[qp];
        __syncwarp();
        window_f32(J, h4, l4, lane, wgt[w], gidx[w]);
        __syncwarp();
        const int Px = J.Pa[0], Py = J.Pa[1], Pz = J.Pa[2], P2 = Py * Pz, R = window_lanes(Py, Pz);
        const size_t JM12 = (size_t)J.M[1] * J.M[2];
        float4* j4 = reinterpret_cast<float4*>(grid + J.grid_off);
        for (int id = lane; id < P2 * R; id += 32) {
            const int xs = id / P2, yz = id - xs * P2, py = yz / Pz, pz = yz - py * Pz;
            const float wyz = wgt[w][1][py] * wgt[w][2][pz];
            const float h0 = fv.x * wyz, h1 = fv.y * wyz, h2 = fv.z * wyz;
            const size_t oyz = (size_t)gidx[w][1][py] * J.M[2] + gidx[w][2][pz];
            for (int px = xs; px < Px; px += R) {
                const float wx = wgt[w][0][px];
                atomicAdd(j4 + (size_t)gidx[w][0][px] * JM12 + oyz, make_float4(h0 * wx, h1 * wx, h2 * wx, 0.f));
            }
        }
    }
}

// Gathering, one target per warp: the target's window is walked with lanes
// over its (y, z) points and a loop over x.  Each axis' weights and wrapped
// grid offsets (32-bit element offsets: x M_y M_z, y M_z, z) are laid out in
// the warp's shared rows once, so the inner loop is one broadcast shared
// load, one integer add, one 16-byte grid load and three FMAs per point; x
// rows are summed in plain FP32 (<= 32 same-sign-weighted terms) and rows
// Kahan-summed.  The weights come from the FP32 window of the point-wise
// spreading kernel (window_f32).  Grids of up to 1024^3 points keep the
// offsets below 2^31.
__global__ void __launch_bounds__(kSpreadWarps * 32)
    k_gather_f4t(const PbInst* __restrict__ inst, const int* __restrict__ ntot_p, const float4* __restrict__ pa,
                 const float4* __restrict__ pb, const float* __restrict__ grid, float* __restrict__ u_k)
{
    __shared__ float2 xw[kSpreadWarps][kMaxP];  // x: (weight, offset bits)
    __shared__ float2 yw[kSpreadWarps][kMaxP];  // y: (weight, offset bits)
    __shared__ float2 zw[kSpreadWarps][kMaxP];  // z: (weight, offset bits)
    const int ntot = *ntot_p;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int s = blockIdx.x * kSpreadWarps + w;
    if (s >= ntot) return;
    const float4 h4 = pa[s], l4 = pb[s];
    const PbInst& I = inst[__float_as_int(h4.w)];
    int g0 = 0;
    float base = 0.f;
    if (lane < 3) {  // the cell and the offset from the window start, as window_f32
        const float xh = lane == 0 ? h4.x : lane == 1 ? h4.y : h4.z;
        const float xl = lane == 0 ? l4.x : lane == 1 ? l4.y : l4.z;
        const float gi = I.gihf[lane];
        const int c = min(max((int)floorf(fmaf(xh, gi, xl * gi)), 0), I.M[lane] - 1);
        g0 = c - I.Pa[lane] / 2 + 1;
        const float gf = (float)g0, hh = I.ghh[lane];
        const float p = gf * hh, e = fmaf(gf, hh, -p);  // g0 hh = p + e exactly
        base = ((xh - p) - e) + (xl - gf * I.ghl[lane]);
    }
    const float inv_eta = I.inv_eta_f;
    const int stride[3] = {I.M[1] * I.M[2], I.M[2], 1};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int ga = __shfl_sync(kFull, g0, a);
        const float ba = __shfl_sync(kFull, base, a);
        if (lane < I.Pa[a]) {
            const float dx = fmaf(-(float)lane, I.ghh[a], ba);
            const float2 v = make_float2(expf(-dx * dx * inv_eta),
                                         __int_as_float(((ga + lane) & (I.M[a] - 1)) * stride[a]));
            if (a == 0)
                xw[w][lane] = v;
            else if (a == 1)
                yw[w][lane] = v;
            else
                zw[w][lane] = v;
        }
    }
    __syncwarp();
    const int Px = I.Pa[0], Py = I.Pa[1], Pz = I.Pa[2], P2 = Py * Pz;
    const unsigned inv_pz = ((1u << 20) + Pz - 1) / Pz;  // exact quotients for yz < 2^15
    const float4* g4 = reinterpret_cast<const float4*>(grid + I.grid_off);
    float s0 = 0, s1 = 0, s2 = 0, c0 = 0, c1 = 0, c2 = 0;
    for (int yz = lane; yz < P2; yz += 32) {
        const int py = (int)(((unsigned)yz * inv_pz) >> 20), pz = yz - py * Pz;
        const float2 ey = yw[w][py], ez = zw[w][pz];
        const int oyz = __float_as_int(ey.y) + __float_as_int(ez.y);
        const float4* row = g4 + oyz;
        float r0 = 0, r1 = 0, r2 = 0;
#pragma unroll 4
        for (int px = 0; px < Px; px++) {
            const float2 ex = xw[w][px];
            const float4 v = __ldg(row + __float_as_int(ex.y));
            r0 = fmaf(ex.x, v.x, r0);
            r1 = fmaf(ex.x, v.y, r1);
            r2 = fmaf(ex.x, v.z, r2);
        }
        const float wyz = ey.x * ez.x;
        kahan_add(s0, c0, wyz * r0);
        kahan_add(s1, c1, wyz * r1);
        kahan_add(s2, c2, wyz * r2);
    }
    s0 -= c0;
    s1 -= c1;
    s2 -= c2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s0 += __shfl_xor_sync(kFull, s0, o);
        s1 += __shfl_xor_sync(kFull, s1, o);
        s2 += __shfl_xor_sync(kFull, s2, o);
    }
    if (lane == 0) {
        u_k[3 * (size_t)s] = s0;
        u_k[3 * (size_t)s + 1] = s1;
        u_k[3 * (size_t)s + 2] = s2;
    }
}

template <class T>
void launch_spread(const PbInst* inst, int ninst, const int* src_offsets, int ncap, const void* pos_a,
                   const void* pos_b, const void* frc, T* grid, cudaStream_t s)
{
    if (ncap <= 0) return;
    int blocks = (ncap + 63 + kSpreadWarps - 1) / kSpreadWarps;  // spread_order covers up to 64 R >= ntot
    const int* ntot = src_offsets + ninst;
    if (sizeof(T) == 4) {
        const int ng = (ncap + kSpreadGroup - 1) / kSpreadGroup;
        k_spread_f4g<<<(ng + 63 + kSpreadWarps - 1) / kSpreadWarps, kSpreadWarps * 32, 0, s>>>(
            inst, ntot, (const float4*)pos_a, (const float4*)pos_b, (const float4*)frc, (float*)grid);
    }
    else
        k_spread<T, Dbl4, Dbl4><<<blocks, kSpreadWarps * 32, 0, s>>>(
            inst, ntot, (const Dbl4*)pos_a, (const Dbl4*)pos_b, (const Dbl4*)frc, grid);
}

template <class T>
void launch_gather(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const void* pos_a,
                   const void* pos_b, const T* grid, T* u_k, cudaStream_t s)
{
    if (ncap <= 0) return;
    int blocks = (ncap + kSpreadWarps - 1) / kSpreadWarps;
    const int* ntot = tgt_offsets + ninst;
    if (sizeof(T) == 4)
        k_gather_f4t<<<(ncap + kSpreadWarps - 1) / kSpreadWarps, kSpreadWarps * 32, 0, s>>>(
            inst, ntot, (const float4*)pos_a, (const float4*)pos_b, (const float*)grid, (float*)u_k);
    else
        k_gather<T, Dbl4><<<blocks, kSpreadWarps * 32, 0, s>>>(inst, ntot, (const Dbl4*)pos_a,
                                                                    (const Dbl4*)pos_b, grid, u_k);
}

// Clears the grids of the instances that have sources or targets (a capacity
// plan's unused positions are left alone): 4 M^3 elements of esz bytes each.
__global__ void k_zero_grids(const PbInst* __restrict__ inst, char* __restrict__ grid, int esz)
{
    const PbInst& I = inst[blockIdx.y];
    if (I.n_src == 0 && I.n_tgt == 0) return;
    const size_t n16 = (size_t)I.M[0] * I.M[1] * I.M[2] * 4 * esz / 16;
    float4* g = reinterpret_cast<float4*>(grid + (size_t)I.grid_off * esz);
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
        g[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

void launch_zero_grids(const PbInst* inst, int ninst, void* grid, int esz, cudaStream_t s)
{
    if (ninst <= 0) return;
    k_zero_grids<<<dim3(256, (unsigned)ninst), 256, 0, s>>>(inst, (char*)grid, esz);
}

template void launch_spread<float>(const PbInst*, int, const int*, int, const void*, const void*, const void*, float*,
                                   cudaStream_t);
template void launch_spread<double>(const PbInst*, int, const int*, int, const void*, const void*, const void*,
                                    double*, cudaStream_t);
template void launch_gather<float>(const PbInst*, int, const int*, int, const void*, const void*, const float*,
                                   float*, cudaStream_t);
template void launch_gather<double>(const PbInst*, int, const int*, int, const void*, const void*, const double*,
                                    double*, cudaStream_t);

// ---------------------------------------------------------------------------
// Shared-memory Stockham FFT (radix 4, with one radix-2 stage when log2 N is odd)
// ---------------------------------------------------------------------------
// Transforms `nl` lines of length N held in smem: element (l, i) at
// buf[l*ls + i*es].  Forward uses W_N^k = exp(-2 pi i k/N) from tw[k] (k < N/2);
// inverse conjugates.  Unnormalised.  Returns the buffer holding the result.
// Thread mapping: `lfast` puts the line index in the fastest thread dimension
// (use when es == 1 is false, i.e. lines interleaved).  Stage with sub-size Ns
// (autosort): inputs j + r N/R, twiddles W_{R Ns}^{r k} (k = j mod Ns), output
// (j - k) R + k + r Ns.
template <class T2>
__device__ T2* stockham(T2* a, T2* b, int N, int nl, int ls, int es, const T2* __restrict__ tw, bool inverse,
                        bool lfast)
{
    int lgN = 0;
    while ((1 << lgN) < N) lgN++;
    const float inv_nl = 1.0f / (float)nl;
    int Ns = 1;
    if (lgN & 1) {  // radix 2 (no twiddles at Ns = 1)
        const int half = N >> 1, total = nl * half;
        for (int wdx = threadIdx.x; wdx < total; wdx += blockDim.x) {
            int l, j;
            if (lfast) {
                j = __float2int_rz(((float)wdx + 0.5f) * inv_nl);
                l = wdx - j * nl;
            } else {
                j = wdx & (half - 1);
                l = wdx >> (lgN - 1);
            }
            const T2 a0 = a[l * ls + j * es], a1 = a[l * ls + (j + half) * es];
            T2 s0, d0;
            s0.x = a0.x + a1.x;
            s0.y = a0.y + a1.y;
            d0.x = a0.x - a1.x;
            d0.y = a0.y - a1.y;
            b[l * ls + (2 * j) * es] = s0;
            b[l * ls + (2 * j + 1) * es] = d0;
        }
        __syncthreads();
        T2* t = a;
        a = b;
        b = t;
        Ns = 2;
    }
    const int quarter = N >> 2, total = nl * quarter;
    for (; Ns < N; Ns <<= 2) {
        const int tstep = N / (4 * Ns);
        for (int wdx = threadIdx.x; wdx < total; wdx += blockDim.x) {
            int l, j;
            if (lfast) {
                j = __float2int_rz(((float)wdx + 0.5f) * inv_nl);
                l = wdx - j * nl;
            } else {
                j = wdx & (quarter - 1);
                l = wdx >> (lgN - 2);
            }
            T2 v0 = a[l * ls + j * es], v1 = a[l * ls + (j + quarter) * es], v2 = a[l * ls + (j + 2 * quarter) * es],
               v3 = a[l * ls + (j + 3 * quarter) * es];
            const int k = j & (Ns - 1);
            if (Ns > 1) {
                T2 w1 = tw[k * tstep];
                if (inverse) w1.y = -w1.y;
                const T2 w2 = cmul(w1, w1), w3 = cmul(w2, w1);
                v1 = cmul(v1, w1);
                v2 = cmul(v2, w2);
                v3 = cmul(v3, w3);
            }
            T2 t0, t1, t2, t3;
            t0.x = v0.x + v2.x;
            t0.y = v0.y + v2.y;
            t1.x = v0.x - v2.x;
            t1.y = v0.y - v2.y;
            t2.x = v1.x + v3.x;
            t2.y = v1.y + v3.y;
            // t3 = (v1 - v3) * (-i) forward, * (+i) inverse
            const decltype(v1.x) ex = v1.x - v3.x, ey = v1.y - v3.y;
            if (inverse) {
                t3.x = -ey;
                t3.y = ex;
            } else {
                t3.x = ey;
                t3.y = -ex;
            }
            const int o = l * ls + (((j - k) << 2) + k) * es;
            T2 X;
            X.x = t0.x + t2.x;
            X.y = t0.y + t2.y;
            b[o] = X;
            X.x = t1.x + t3.x;
            X.y = t1.y + t3.y;
            b[o + Ns * es] = X;
            X.x = t0.x - t2.x;
            X.y = t0.y - t2.y;
            b[o + 2 * Ns * es] = X;
            X.x = t1.x - t3.x;
            X.y = t1.y - t3.y;
            b[o + 3 * Ns * es] = X;
        }
        __syncthreads();
        T2* t = a;
        a = b;
        b = t;
    }
    return a;
}

// Twiddle table layout for one grid bucket (M = {Mx, My, Mz}, Nh = Mz/2):
//   [W_Nh: Nh/2][W_My: My/2][W_Mx: Mx/2][R: Nh+1 with R_k = exp(-2 pi i k / Mz)]
struct TwOff {
    int zh, y, x, r, total;
};
__host__ __device__ inline TwOff tw_offsets(const int* M)
{
    TwOff o;
    int Nh = M[2] / 2;
    o.zh = 0;
    o.y = o.zh + (Nh / 2 > 0 ? Nh / 2 : 1);
    o.x = o.y + M[1] / 2;
    o.r = o.x + M[0] / 2;
    o.total = o.r + Nh + 1;
    return o;
}

size_t twiddle_bytes(const int* M, bool fp64)
{
    return (size_t)tw_offsets(M).total * (fp64 ? sizeof(double2) : sizeof(float2));
}

void fill_twiddles(const int* M, bool fp64, void* host_buf)
{
    TwOff o = tw_offsets(M);
    int Nh = M[2] / 2;
    auto put = [&](int at, double ang) {
        double c = cos(ang), s = sin(ang);
        if (fp64) {
            ((double2*)host_buf)[at] = make_double2(c, s);
        } else {
            ((float2*)host_buf)[at] = make_float2((float)c, (float)s);
        }
    };
    for (int k = 0; k < (Nh / 2 > 0 ? Nh / 2 : 1); k++) put(o.zh + k, -2 * kPiD * k / (Nh > 0 ? Nh : 1));
    for (int k = 0; k < M[1] / 2; k++) put(o.y + k, -2 * kPiD * k / M[1]);
    for (int k = 0; k < M[0] / 2; k++) put(o.x + k, -2 * kPiD * k / M[0]);
    for (int k = 0; k <= Nh; k++) put(o.r + k, -2 * kPiD * k / M[2]);
}

// FFT work of a bucket position: a capacity plan (serving slot) keeps room for
// more instances than a batch binds; positions without sources or targets
// are skipped (their grid stays zero, so gathering from it gives zero).
__device__ __forceinline__ bool fft_live(const PbInst* inst, const int* bucket_inst, long long b)
{
    const PbInst& I = inst[bucket_inst[b]];
    return I.n_src > 0 && I.n_tgt > 0;
}

// Planar FP64 grids keep four planes per instance (three components and an
// unused one): grid line of spectrum line L = ((3 b + c) xy + rest).
__device__ __forceinline__ size_t plane_line(long long L, long long xy)
{
    long long v = L / xy, rest = L - v * xy, b = v / 3, c = v - 3 * b;
    return (size_t)((4 * b + c) * xy + rest);
}

// z pass, forward: real lines of length Mz -> Nh+1 complex (packed half-length FFT).
template <class T>
__global__ void k_fft_z_fwd(const T* __restrict__ grid, typename Cx<T>::t* __restrict__ spec, long long nlines, int Mz,
                            int lpb, const typename Cx<T>::t* __restrict__ tw, TwOff o, long long xy,
                            const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    const int Nh = Mz / 2, Mzh = Nh + 1;
    T2* B = A + lpb * Nh;
    long long l0 = (long long)blockIdx.x * lpb;
    int nl = (int)min((long long)lpb, nlines - l0);
    if (!fft_live(inst, bucket_inst, l0 / (3 * xy)) && !fft_live(inst, bucket_inst, (l0 + nl - 1) / (3 * xy))) return;
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, i = idx - l * Nh;
        const T2* src = (const T2*)(grid + plane_line(l0 + l, xy) * Mz);
        A[l * Nh + i] = src[i];
    }
    __syncthreads();
    T2* R = (Nh > 1) ? stockham<T2>(A, B, Nh, nl, Nh, 1, tw + o.zh, false, false) : A;
    const T2* rt = tw + o.r;
    for (int idx = threadIdx.x; idx < nl * Mzh; idx += blockDim.x) {
        int l = idx / Mzh, k = idx - l * Mzh;
        T2 zk = R[l * Nh + (k == Nh ? 0 : k)];
        T2 zm = R[l * Nh + (k == 0 ? 0 : Nh - k)];
        // E = (zk + conj(zm))/2, O = (zk - conj(zm))/(2i)
        T2 E, Od;
        E.x = (T)0.5 * (zk.x + zm.x);
        E.y = (T)0.5 * (zk.y - zm.y);
        Od.x = (T)0.5 * (zk.y + zm.y);
        Od.y = (T)-0.5 * (zk.x - zm.x);
        T2 wo = cmul(rt[k], Od);
        T2 X;
        X.x = E.x + wo.x;
        X.y = E.y + wo.y;
        spec[(size_t)(l0 + l) * Mzh + k] = X;
    }
}

// z pass, inverse: Nh+1 complex -> real line of length Mz.
template <class T>
__global__ void k_fft_z_inv(const typename Cx<T>::t* __restrict__ spec, T* __restrict__ grid, long long nlines, int Mz,
                            int lpb, const typename Cx<T>::t* __restrict__ tw, TwOff o, long long xy,
                            const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    const int Nh = Mz / 2, Mzh = Nh + 1;
    T2* B = A + lpb * Nh;
    const T2* rt = tw + o.r;
    long long l0 = (long long)blockIdx.x * lpb;
    int nl = (int)min((long long)lpb, nlines - l0);
    if (!fft_live(inst, bucket_inst, l0 / (3 * xy)) && !fft_live(inst, bucket_inst, (l0 + nl - 1) / (3 * xy))) return;
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, k = idx - l * Nh;
        const T2* src = spec + (size_t)(l0 + l) * Mzh;
        T2 xk = src[k], xm = src[Nh - k];
        // Z_k = (xk + conj(xm)) + i W^{-k} (xk - conj(xm))
        T2 e, dlt;
        e.x = xk.x + xm.x;
        e.y = xk.y - xm.y;
        dlt.x = xk.x - xm.x;
        dlt.y = xk.y + xm.y;
        T2 wc = rt[k];
        wc.y = -wc.y;
        T2 od = cmul(wc, dlt);
        T2 Z;
        Z.x = e.x - od.y;
        Z.y = e.y + od.x;
        A[l * Nh + k] = Z;
    }
    __syncthreads();
    T2* R = (Nh > 1) ? stockham<T2>(A, B, Nh, nl, Nh, 1, tw + o.zh, true, false) : A;
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, i = idx - l * Nh;
        T2* dst = (T2*)(grid + plane_line(l0 + l, xy) * Mz);
        dst[i] = R[l * Nh + i];
    }
}

// z passes for FP32 grids with interleaved components (float4 per point):
// one grid line (instance, x, y) gives the three spectrum lines of its components.
__global__ void k_fft_z_fwd4(const float4* __restrict__ grid, float2* __restrict__ spec, long long nlines, int Mx,
                             int My, int Mz, int lpb, const float2* __restrict__ tw, TwOff o,
                             const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* A = (float2*)smem_raw;
    const int Nh = Mz / 2, Mzh = Nh + 1;
    float2* B = A + 3 * lpb * Nh;
    long long l0 = (long long)blockIdx.x * lpb;
    int nl = (int)min((long long)lpb, nlines - l0);
    const long long xy_ = (long long)Mx * My;
    if (!fft_live(inst, bucket_inst, l0 / xy_) && !fft_live(inst, bucket_inst, (l0 + nl - 1) / xy_)) return;
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, i = idx - l * Nh;
        const float4* src = grid + (size_t)(l0 + l) * Mz;
        float4 a = src[2 * i], b = src[2 * i + 1];
        A[(3 * l + 0) * Nh + i] = make_float2(a.x, b.x);
        A[(3 * l + 1) * Nh + i] = make_float2(a.y, b.y);
        A[(3 * l + 2) * Nh + i] = make_float2(a.z, b.z);
    }
    __syncthreads();
    float2* R = (Nh > 1) ? stockham<float2>(A, B, Nh, 3 * nl, Nh, 1, tw + o.zh, false, false) : A;
    const float2* rt = tw + o.r;
    const long long xy = (long long)Mx * My;
    for (int idx = threadIdx.x; idx < 3 * nl * Mzh; idx += blockDim.x) {
        int lc = idx / Mzh, k = idx - lc * Mzh;
        int l = lc / 3, c = lc - 3 * l;
        float2 zk = R[lc * Nh + (k == Nh ? 0 : k)];
        float2 zm = R[lc * Nh + (k == 0 ? 0 : Nh - k)];
        float2 E, Od;
        E.x = 0.5f * (zk.x + zm.x);
        E.y = 0.5f * (zk.y - zm.y);
        Od.x = 0.5f * (zk.y + zm.y);
        Od.y = -0.5f * (zk.x - zm.x);
        float2 wo = cmul(rt[k], Od);
        long long line = l0 + l, bi = line / xy, rest = line - bi * xy;
        spec[((size_t)(3 * bi + c) * xy + rest) * Mzh + k] = make_float2(E.x + wo.x, E.y + wo.y);
    }
}

__global__ void k_fft_z_inv4(const float2* __restrict__ spec, float4* __restrict__ grid, long long nlines, int Mx,
                             int My, int Mz, int lpb, const float2* __restrict__ tw, TwOff o,
                             const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* A = (float2*)smem_raw;
    const int Nh = Mz / 2, Mzh = Nh + 1;
    float2* B = A + 3 * lpb * Nh;
    const float2* rt = tw + o.r;
    long long l0 = (long long)blockIdx.x * lpb;
    int nl = (int)min((long long)lpb, nlines - l0);
    if (!fft_live(inst, bucket_inst, l0 / ((long long)Mx * My)) &&
        !fft_live(inst, bucket_inst, (l0 + nl - 1) / ((long long)Mx * My)))
        return;
    const long long xy = (long long)Mx * My;
    for (int idx = threadIdx.x; idx < 3 * nl * Nh; idx += blockDim.x) {
        int lc = idx / Nh, k = idx - lc * Nh;
        int l = lc / 3, c = lc - 3 * l;
        long long line = l0 + l, bi = line / xy, rest = line - bi * xy;
        const float2* src = spec + ((size_t)(3 * bi + c) * xy + rest) * Mzh;
        float2 xk = src[k], xm = src[Nh - k];
        float2 e, dlt;
        e.x = xk.x + xm.x;
        e.y = xk.y - xm.y;
        dlt.x = xk.x - xm.x;
        dlt.y = xk.y + xm.y;
        float2 wc = rt[k];
        wc.y = -wc.y;
        float2 od = cmul(wc, dlt);
        A[lc * Nh + k] = make_float2(e.x - od.y, e.y + od.x);
    }
    __syncthreads();
    float2* R = (Nh > 1) ? stockham<float2>(A, B, Nh, 3 * nl, Nh, 1, tw + o.zh, true, false) : A;
    for (int idx = threadIdx.x; idx < nl * Nh; idx += blockDim.x) {
        int l = idx / Nh, i = idx - l * Nh;
        float2 u0 = R[(3 * l) * Nh + i], u1 = R[(3 * l + 1) * Nh + i], u2 = R[(3 * l + 2) * Nh + i];
        float4* dst = grid + (size_t)(l0 + l) * Mz;
        dst[2 * i] = make_float4(u0.x, u1.x, u2.x, 0.f);
        dst[2 * i + 1] = make_float4(u0.y, u1.y, u2.y, 0.f);
    }
}

// y pass (forward or inverse) over volumes [nvol][Mx][My][Mzh]; tile of TW z' columns.
template <class T>
__global__ void k_fft_y(typename Cx<T>::t* __restrict__ spec, int nvol, int Mx, int My, int Mzh, int TW,
                        const typename Cx<T>::t* __restrict__ tw, int tw_off, bool inverse,
                        const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    T2* B = A + TW * My;
    const int ntile = (Mzh + TW - 1) / TW;
    long long blk = blockIdx.x;
    int tile = (int)(blk % ntile);
    long long vx = blk / ntile;  // vol*Mx + x
    if (!fft_live(inst, bucket_inst, vx / Mx / 3)) return;
    int z0 = tile * TW;
    int nl = min(TW, Mzh - z0);
    T2* base = spec + (size_t)vx * My * Mzh + z0;
    for (int idx = threadIdx.x; idx < My * TW; idx += blockDim.x) {
        int i = idx / TW, l = idx - i * TW;
        if (l < nl) A[i * TW + l] = base[(size_t)i * Mzh + l];
    }
    __syncthreads();
    T2* R = stockham<T2>(A, B, My, TW, 1, TW, tw + tw_off, inverse, true);
    for (int idx = threadIdx.x; idx < My * TW; idx += blockDim.x) {
        int i = idx / TW, l = idx - i * TW;
        if (l < nl) base[(size_t)i * Mzh + l] = R[i * TW + l];
    }
}

// x pass fused: forward FFT along x of the three components, Green tensor
// multiply, inverse FFT along x.  One block per (instance, y, z'-tile).
struct GreenConst {
    double twopi_L[3];
    double a2, a1_over_a2, gexp, kfac;  // kfac * (1 + a1 k^2/a^2) exp(-k^2 gexp) / (k^2 (k^2 + a^2))
};

template <class T>
__global__ void k_fft_x_green(typename Cx<T>::t* __restrict__ spec, const PbInst* __restrict__ inst,
                              const int* __restrict__ bucket_inst, long long base_off, int Mx, int My, int Mzh, int Mz,
                              int TW, const typename Cx<T>::t* __restrict__ tw, int tw_off)
{
    typedef typename Cx<T>::t T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2* A = (T2*)smem_raw;
    T2* B = A + 3 * TW * Mx;
    const int ntile = (Mzh + TW - 1) / TW;
    long long blk = blockIdx.x;
    int tile = (int)(blk % ntile);
    long long r = blk / ntile;
    int y = (int)(r % My);
    int qi = (int)(r / My);
    if (!fft_live(inst, bucket_inst, qi)) return;
    const PbInst& I = inst[bucket_inst[qi]];
    int z0 = tile * TW;
    int nl = min(TW, Mzh - z0);
    const size_t vol = (size_t)Mx * My * Mzh;
    T2* base = spec + (I.spec_off - base_off) + (size_t)y * Mzh + z0;
    // smem layout: line (c, l) at (c*TW + l), element i stride 3*TW
    const int NL = 3 * TW;
    for (int idx = threadIdx.x; idx < 3 * Mx * TW; idx += blockDim.x) {
        int l = idx % TW, rest = idx / TW, i = rest % Mx, c = rest / Mx;
        if (l < nl) A[i * NL + c * TW + l] = base[c * vol + (size_t)i * My * Mzh + l];
    }
    __syncthreads();
    T2* R = stockham<T2>(A, B, Mx, NL, 1, NL, tw + tw_off, false, true);
    T2* S = (R == A) ? B : A;
    // Green multiply in place in R
    const double tpx = 2 * kPiD / I.L[0], tpy = 2 * kPiD / I.L[1], tpz = 2 * kPiD / I.L[2];
    const double a2 = I.alpha * I.alpha;
    const T a1oa2 = (T)(-expm1(-a2 * I.d * I.d / 4) / a2);
    const T gexp = (T)(I.d * I.d / 4 - I.eta / 2);
    const T kfac = (T)I.kfac;
    const int My_ = My;
    int ny = (y < My_ / 2) ? y : y - My_;
    bool ynyq = (2 * y == My_);
    for (int idx = threadIdx.x; idx < Mx * TW; idx += blockDim.x) {
        int l = idx % TW, i = idx / TW;
        if (l >= nl) continue;
        int kz = z0 + l;
        int nx = (i < Mx / 2) ? i : i - Mx;
        bool zero = (2 * i == Mx) || ynyq || (2 * kz == Mz) || (nx == 0 && ny == 0 && kz == 0);
        T2* v0 = &R[i * NL + 0 * TW + l];
        T2* v1 = &R[i * NL + 1 * TW + l];
        T2* v2 = &R[i * NL + 2 * TW + l];
        if (zero) {
            *v0 = T2{0, 0};
            *v1 = T2{0, 0};
            *v2 = T2{0, 0};
            continue;
        }
        T kx = (T)tpx * (T)nx, ky = (T)tpy * (T)ny, kzv = (T)tpz * (T)kz;  // in T: no FP64 work on FP32 grids
        T kn = kx * kx + ky * ky + kzv * kzv;
        T s = kfac * ((T)1 + a1oa2 * kn) * exp(-kn * gexp) / (kn * (kn + (T)a2));
        T2 A0 = *v0, A1 = *v1, A2 = *v2;
        T dr = kx * A0.x + ky * A1.x + kzv * A2.x;
        T di = kx * A0.y + ky * A1.y + kzv * A2.y;
        *v0 = T2{s * (kn * A0.x - kx * dr), s * (kn * A0.y - kx * di)};
        *v1 = T2{s * (kn * A1.x - ky * dr), s * (kn * A1.y - ky * di)};
        *v2 = T2{s * (kn * A2.x - kzv * dr), s * (kn * A2.y - kzv * di)};
    }
    __syncthreads();
    T2* R2 = stockham<T2>(R, S, Mx, NL, 1, NL, tw + tw_off, true, true);
    for (int idx = threadIdx.x; idx < 3 * Mx * TW; idx += blockDim.x) {
        int l = idx % TW, rest = idx / TW, i = rest % Mx, c = rest / Mx;
        if (l < nl) base[c * vol + (size_t)i * My * Mzh + l] = R2[i * NL + c * TW + l];
    }
}

// ---------------------------------------------------------------------------
// Register FFT passes (FP32 grids, line lengths 4..256)
// ---------------------------------------------------------------------------
// A line of length N = N1 N2 is transformed by T threads, each holding N/T
// values in registers: N2 FFTs of length N1 over x[N2 n1 + n2] (thread t takes
// n2 = t, t + T, ...), the twiddles W_N^(n2 k1), one exchange through shared
// memory, then N1 FFTs of length N2 (thread t takes k1 = t, t + T, ...); the
// result X[k1 + N1 k2] stays in the registers of the thread that owns k1.
// Lengths up to 16 are radix-2 butterflies on named registers with constant
// twiddles.  Forward uses W = exp(-2 pi i / N), inverse its conjugate, both
// unnormalised, as the shared-memory passes above.

// cos and sin of 2 pi m / 16
__host__ __device__ constexpr float c16(int m)
{
    return m == 0 ? 1.f : m == 1 ? 0.92387953251128674f : m == 2 ? 0.70710678118654752f
         : m == 3 ? 0.38268343236508977f : m == 4 ? 0.f : m == 5 ? -0.38268343236508977f
         : m == 6 ? -0.70710678118654752f : -0.92387953251128674f;
}
__host__ __device__ constexpr float s16(int m)
{
    return m == 0 ? 0.f : m == 1 ? 0.38268343236508977f : m == 2 ? 0.70710678118654752f
         : m == 3 ? 0.92387953251128674f : m == 4 ? 1.f : m == 5 ? 0.92387953251128674f
         : m == 6 ? 0.70710678118654752f : 0.38268343236508977f;
}

// x * W_16^m (m < 8 and known at compile time after unrolling)
template <bool INV>
__device__ __forceinline__ float2 w16_mul(float2 x, int m)
{
    if (m == 0) return x;
    if (m == 4) return INV ? make_float2(-x.y, x.x) : make_float2(x.y, -x.x);
    const float c = c16(m), s = INV ? s16(m) : -s16(m);
    return make_float2(fmaf(x.x, c, -x.y * s), fmaf(x.x, s, x.y * c));
}

__host__ __device__ constexpr int bitrev(int i, int bits)
{
    int r = 0;
    for (int b = 0; b < bits; b++) r |= ((i >> b) & 1) << (bits - 1 - b);
    return r;
}
__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }

// In-register FFT of R <= 16 values, natural order in and out.
template <int R, bool INV>
__device__ __forceinline__ void fft_reg(float2 (&v)[R])
{
    constexpr int L = ilog2(R);
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int j = bitrev(i, L);
        if (j > i) {
            const float2 t = v[i];
            v[i] = v[j];
            v[j] = t;
        }
    }
#pragma unroll
    for (int h = 1; h < R; h <<= 1) {
#pragma unroll
        for (int k = 0; k < h; k++) {
            const int m = k * (8 / h);  // W_{2h}^k = W_16^(8 k / h)
#pragma unroll
            for (int j = k; j < R; j += 2 * h) {
                const float2 b = w16_mul<INV>(v[j + h], m), a = v[j];
                v[j] = make_float2(a.x + b.x, a.y + b.y);
                v[j + h] = make_float2(a.x - b.x, a.y - b.y);
            }
        }
    }
}

// x * W_N^m from the table of W_N^k, k < N/2 (conjugated for the inverse)
template <bool INV>
__device__ __forceinline__ float2 twN_mul(float2 x, int m, int N, const float2* __restrict__ tw)
{
    const int h = N >> 1;
    float2 w = __ldg(tw + (m < h ? m : m - h));
    if (m >= h) w = make_float2(-w.x, -w.y);
    if (INV) w.y = -w.y;
    return cmul(x, w);
}

// Four-step line transform: A (stage-1 layout, A[a][n1] = x[N2 n1 + t + T a]) ->
// B (stage-2 layout, B[b][k2] = X[t + T b + N1 k2]).  `ex` holds N elements of
// this line at stride LS (ex[e * LS]); the caller synchronises before the
// exchange buffer is reused.
// Shared-memory slot of element e of a line: ex[e * LS] for the passes
// whose lines sit in the lanes of a warp (y, x); for the z passes, where a
// warp holds 32/T lines times the T threads of each, the line index `ll` is
// rotated within its aligned group of 32 by (32/T) ((e + e/N1) mod T), so
// that the T threads of a line, which differ in n2 (stage 1) or in k1
// (stage 2), hit different banks.
template <int T, int N1>
__device__ __forceinline__ int zslot(int e, int ll, int LS)
{
    const int s = (e + e / N1) & (T - 1);
    return e * LS + (ll & ~31) + ((ll + (32 / T) * s) & 31);
}

template <int N1, int N2, int T, bool INV, bool ZSW = false>
__device__ __forceinline__ void line_fft(float2 (&A)[N2 / T][N1], float2 (&B)[N1 / T][N2], float2* ex, int LS, int t,
                                         const float2* __restrict__ tw, int ll = 0)
{
    constexpr int N = N1 * N2;
#pragma unroll
    for (int a = 0; a < N2 / T; a++) {
        fft_reg<N1, INV>(A[a]);
        const int n2 = t + T * a;
        if (N2 > 1) {
#pragma unroll
            for (int k1 = 1; k1 < N1; k1++) A[a][k1] = twN_mul<INV>(A[a][k1], n2 * k1, N, tw);
        }
    }
    if constexpr (N2 == 1) {
#pragma unroll
        for (int b = 0; b < N1 / T; b++) B[b][0] = A[0][b];
    } else {
#pragma unroll
        for (int a = 0; a < N2 / T; a++) {
            const int n2 = t + T * a;
#pragma unroll
            for (int k1 = 0; k1 < N1; k1++) {
                const int e = n2 * N1 + k1;
                ex[ZSW ? zslot<T, N1>(e, ll, LS) : e * LS] = A[a][k1];
            }
        }
        __syncthreads();
#pragma unroll
        for (int b = 0; b < N1 / T; b++) {
            const int k1 = t + T * b;
#pragma unroll
            for (int n2 = 0; n2 < N2; n2++) {
                const int e = n2 * N1 + k1;
                B[b][n2] = ex[ZSW ? zslot<T, N1>(e, ll, LS) : e * LS];
            }
            fft_reg<N2, INV>(B[b]);
        }
    }
}

// y pass: lines along y (stride Mzh) of the spectrum volumes; a block is 32
// consecutive z' lines (lanes) times T threads per line (warps).
template <int N1, int N2, int T, bool INV>
__global__ void __launch_bounds__(32 * T)
    k_fft_y_reg(float2* __restrict__ spec, int Mx, int Mzh, const float2* __restrict__ tw,
                const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst)
{
    constexpr int N = N1 * N2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* ex = (float2*)smem_raw;
    const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
    const int nz = Mzh - 1;  // the z Nyquist plane is zeroed by the Green multiply: not transformed
    const int ntile = (nz + 31) >> 5;
    const long long blk = blockIdx.x;
    const int tile = (int)(blk % ntile);
    const long long vx = blk / ntile;  // volume * Mx + x
    if (!fft_live(inst, bucket_inst, vx / Mx / 3)) return;
    const int z = tile * 32 + lane;
    const bool ok = z < nz;
    float2* base = spec + (size_t)vx * N * Mzh + (ok ? z : 0);
    float2 A[N2 / T][N1], B[N1 / T][N2];
#pragma unroll
    for (int a = 0; a < N2 / T; a++)
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++)
            A[a][n1] = ok ? base[(size_t)(N2 * n1 + t + T * a) * Mzh] : make_float2(0.f, 0.f);
    line_fft<N1, N2, T, INV>(A, B, ex + lane, 32, t, tw);
#pragma unroll
    for (int b = 0; b < N1 / T; b++)
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++)
            if (ok) base[(size_t)(t + T * b + N1 * k2) * Mzh] = B[b][k2];
}

// x pass fused with the Green multiply: for 32 consecutive z' lines of one
// (instance, y), the three components' forward x transforms are kept in
// shared memory (SP[c][k][line]), multiplied by the Green tensor and
// transformed back.  The Green multiply is the one of k_fft_x_green.
template <int N1, int N2, int T>
__global__ void __launch_bounds__(32 * T)
    k_fft_x_green_reg(float2* __restrict__ spec, const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst,
                      long long base_off, int My, int Mzh, int Mz, const float2* __restrict__ tw)
{
    constexpr int N = N1 * N2;  // Mx
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* SP = (float2*)smem_raw;  // [3][N][32]
    const int lane = threadIdx.x & 31, t = threadIdx.x >> 5;
    const int nz = Mzh - 1;  // z' < Mz/2; the Nyquist plane z' = Mz/2 is zero after the Green multiply
    const int ntile = (nz + 31) >> 5;
    const long long blk = blockIdx.x;
    const int tile = (int)(blk % ntile);
    const long long r = blk / ntile;
    const int y = (int)(r % My);
    const int qi = (int)(r / My);
    if (!fft_live(inst, bucket_inst, qi)) return;
    const PbInst& I = inst[bucket_inst[qi]];
    const int z = tile * 32 + lane;
    const bool ok = z < nz;
    const size_t vol = (size_t)N * My * Mzh, xs = (size_t)My * Mzh;
    float2* base = spec + (I.spec_off - base_off) + (size_t)y * Mzh + (ok ? z : 0);
    if (tile == 0) {  // the Nyquist line of this (instance, y), for the inverse y and z passes
        float2* nyq = spec + (I.spec_off - base_off) + (size_t)y * Mzh + nz;
        for (int i = threadIdx.x; i < 3 * N; i += 32 * T)
            nyq[(size_t)(i / N) * vol + (size_t)(i % N) * xs] = make_float2(0.f, 0.f);
    }
    float2 A[N2 / T][N1], B[N1 / T][N2];
#pragma unroll 1
    for (int c = 0; c < 3; c++) {
        float2* ex = SP + (size_t)c * N * 32 + lane;
#pragma unroll
        for (int a = 0; a < N2 / T; a++)
#pragma unroll
            for (int n1 = 0; n1 < N1; n1++)
                A[a][n1] = ok ? base[c * vol + (size_t)(N2 * n1 + t + T * a) * xs] : make_float2(0.f, 0.f);
        line_fft<N1, N2, T, false>(A, B, ex, 32, t, tw);
        __syncthreads();
#pragma unroll
        for (int b = 0; b < N1 / T; b++)
#pragma unroll
            for (int k2 = 0; k2 < N2; k2++) ex[(size_t)(t + T * b + N1 * k2) * 32] = B[b][k2];
    }
    __syncthreads();
    // Green multiply (as k_fft_x_green, in FP32)
    {
        const float tpx = (float)(2 * kPiD / I.L[0]), tpy = (float)(2 * kPiD / I.L[1]),
                    tpz = (float)(2 * kPiD / I.L[2]);
        const double a2d = I.alpha * I.alpha;
        const float a2 = (float)a2d;
        const float a1oa2 = (float)(-expm1(-a2d * I.d * I.d / 4) / a2d);
        const float gexp = (float)(I.d * I.d / 4 - I.eta / 2);
        const float kfac = (float)I.kfac;
        const int ny = (y < My / 2) ? y : y - My;
        const bool ynyq = (2 * y == My);
        const float ky = tpy * (float)ny, kzv = tpz * (float)z;
#pragma unroll 4
        for (int i = t; i < N; i += T) {
            float2* v0 = SP + (size_t)i * 32 + lane;
            float2* v1 = v0 + (size_t)N * 32;
            float2* v2 = v1 + (size_t)N * 32;
            const int nx = (i < N / 2) ? i : i - N;
            const bool zero = (2 * i == N) || ynyq || (2 * z == Mz) || (nx == 0 && ny == 0 && z == 0);
            if (zero) {
                *v0 = make_float2(0.f, 0.f);
                *v1 = make_float2(0.f, 0.f);
                *v2 = make_float2(0.f, 0.f);
                continue;
            }
            const float kx = tpx * (float)nx;
            const float kn = kx * kx + ky * ky + kzv * kzv;
            const float sc = kfac * (1.f + a1oa2 * kn) * expf(-kn * gexp) / (kn * (kn + a2));
            const float2 A0 = *v0, A1 = *v1, A2 = *v2;
            const float dr = kx * A0.x + ky * A1.x + kzv * A2.x;
            const float di = kx * A0.y + ky * A1.y + kzv * A2.y;
            *v0 = make_float2(sc * (kn * A0.x - kx * dr), sc * (kn * A0.y - kx * di));
            *v1 = make_float2(sc * (kn * A1.x - ky * dr), sc * (kn * A1.y - ky * di));
            *v2 = make_float2(sc * (kn * A2.x - kzv * dr), sc * (kn * A2.y - kzv * di));
        }
    }
    __syncthreads();
#pragma unroll 1
    for (int c = 0; c < 3; c++) {
        float2* ex = SP + (size_t)c * N * 32 + lane;
#pragma unroll
        for (int a = 0; a < N2 / T; a++)
#pragma unroll
            for (int n1 = 0; n1 < N1; n1++) A[a][n1] = ex[(size_t)(N2 * n1 + t + T * a) * 32];
        __syncthreads();
        line_fft<N1, N2, T, true>(A, B, ex, 32, t, tw);
#pragma unroll
        for (int b = 0; b < N1 / T; b++)
#pragma unroll
            for (int k2 = 0; k2 < N2; k2++)
                if (ok) base[c * vol + (size_t)(t + T * b + N1 * k2) * xs] = B[b][k2];
    }
}

// z pass, forward, FP32 float4 grid lines (instance, x, y) of length Mz = 2 Nh:
// the packed half-length transform of the three components, then the split
// into the Nh + 1 half-spectrum values of each.  256 threads: 256 / T lines.
template <int N1, int N2, int T>
__global__ void __launch_bounds__(256)
    k_fft_z_fwd_reg(const float4* __restrict__ grid, float2* __restrict__ spec, long long nlines, int Mx, int My,
                    const float2* __restrict__ tw, const float2* __restrict__ rt, const PbInst* __restrict__ inst,
                    const int* __restrict__ bucket_inst)
{
    constexpr int Nh = N1 * N2, Mzh = Nh + 1, LPC = 256 / T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* ex = (float2*)smem_raw;  // [3][Nh][LPC]
    const int t = threadIdx.x % T, ll = threadIdx.x / T;
    const long long l0 = (long long)blockIdx.x * LPC;
    const long long xy = (long long)Mx * My;
    const long long lastl = min(l0 + LPC, nlines) - 1;
    if (!fft_live(inst, bucket_inst, l0 / xy) && !fft_live(inst, bucket_inst, lastl / xy)) return;
    const long long line = l0 + ll;
    const bool ok = line < nlines;
    const float4* src = grid + (size_t)(ok ? line : 0) * (2 * Nh);
    float2 A0[N2 / T][N1], A1[N2 / T][N1], A2[N2 / T][N1];
#pragma unroll
    for (int a = 0; a < N2 / T; a++)
#pragma unroll
        for (int n1 = 0; n1 < N1; n1++) {
            const int n = N2 * n1 + t + T * a;
            const float4 p = ok ? src[2 * n] : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 q = ok ? src[2 * n + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
            A0[a][n1] = make_float2(p.x, q.x);
            A1[a][n1] = make_float2(p.y, q.y);
            A2[a][n1] = make_float2(p.z, q.z);
        }
    float2 B0[N1 / T][N2], B1[N1 / T][N2], B2[N1 / T][N2];
    line_fft<N1, N2, T, false, true>(A0, B0, ex, LPC, t, tw, ll);
    line_fft<N1, N2, T, false, true>(A1, B1, ex + (size_t)Nh * LPC, LPC, t, tw, ll);
    line_fft<N1, N2, T, false, true>(A2, B2, ex + (size_t)2 * Nh * LPC, LPC, t, tw, ll);
    __syncthreads();
#pragma unroll
    for (int b = 0; b < N1 / T; b++)
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) {
            const int k = t + T * b + N1 * k2, o = zslot<T, N1>(k, ll, LPC);
            ex[o] = B0[b][k2];
            ex[(size_t)Nh * LPC + o] = B1[b][k2];
            ex[(size_t)2 * Nh * LPC + o] = B2[b][k2];
        }
    __syncthreads();
    if (!ok) return;
    const long long bi = line / xy, rest = line - bi * xy;
    for (int k = t; k < Mzh; k += T) {
        const float2 w = __ldg(rt + k);
        const int ok_ = zslot<T, N1>(k == Nh ? 0 : k, ll, LPC), om = zslot<T, N1>(k == 0 ? 0 : Nh - k, ll, LPC);
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const float2* Z = ex + (size_t)c * Nh * LPC;
            const float2 zk = Z[ok_];
            const float2 zm = Z[om];
            const float2 E = make_float2(0.5f * (zk.x + zm.x), 0.5f * (zk.y - zm.y));
            const float2 Od = make_float2(0.5f * (zk.y + zm.y), -0.5f * (zk.x - zm.x));
            const float2 wo = cmul(w, Od);
            spec[((size_t)(3 * bi + c) * xy + rest) * Mzh + k] = make_float2(E.x + wo.x, E.y + wo.y);
        }
    }
}

// z pass, inverse: Nh + 1 half-spectrum values of each component -> one real
// float4 grid line (three components interleaved, fourth zero).
template <int N1, int N2, int T>
__global__ void __launch_bounds__(256)
    k_fft_z_inv_reg(const float2* __restrict__ spec, float4* __restrict__ grid, long long nlines, int Mx, int My,
                    const float2* __restrict__ tw, const float2* __restrict__ rt, const PbInst* __restrict__ inst,
                    const int* __restrict__ bucket_inst)
{
    constexpr int Nh = N1 * N2, Mzh = Nh + 1, LPC = 256 / T;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* ex = (float2*)smem_raw;  // [3][Nh][LPC]
    const int t = threadIdx.x % T, ll = threadIdx.x / T;
    const long long l0 = (long long)blockIdx.x * LPC;
    const long long xy = (long long)Mx * My;
    const long long lastl = min(l0 + LPC, nlines) - 1;
    if (!fft_live(inst, bucket_inst, l0 / xy) && !fft_live(inst, bucket_inst, lastl / xy)) return;
    const long long line = l0 + ll;
    const bool ok = line < nlines;
    const long long bi = (ok ? line : 0) / xy, rest = (ok ? line : 0) - bi * xy;
    float2 A[3][N2 / T][N1];
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float2* src = spec + ((size_t)(3 * bi + c) * xy + rest) * Mzh;
#pragma unroll
        for (int a = 0; a < N2 / T; a++)
#pragma unroll
            for (int n1 = 0; n1 < N1; n1++) {
                const int k = N2 * n1 + t + T * a;
                float2 Z = make_float2(0.f, 0.f);
                if (ok) {
                    const float2 xk = src[k], xm = src[Nh - k];
                    const float2 e = make_float2(xk.x + xm.x, xk.y - xm.y);
                    const float2 dlt = make_float2(xk.x - xm.x, xk.y + xm.y);
                    float2 wc = __ldg(rt + k);
                    wc.y = -wc.y;
                    const float2 od = cmul(wc, dlt);
                    Z = make_float2(e.x - od.y, e.y + od.x);
                }
                A[c][a][n1] = Z;
            }
    }
    float2 B0[N1 / T][N2], B1[N1 / T][N2], B2[N1 / T][N2];
    line_fft<N1, N2, T, true, true>(A[0], B0, ex, LPC, t, tw, ll);
    line_fft<N1, N2, T, true, true>(A[1], B1, ex + (size_t)Nh * LPC, LPC, t, tw, ll);
    line_fft<N1, N2, T, true, true>(A[2], B2, ex + (size_t)2 * Nh * LPC, LPC, t, tw, ll);
    if (!ok) return;
    float4* dst = grid + (size_t)line * (2 * Nh);
#pragma unroll
    for (int b = 0; b < N1 / T; b++)
#pragma unroll
        for (int k2 = 0; k2 < N2; k2++) {
            const int k = t + T * b + N1 * k2;
            dst[2 * k] = make_float4(B0[b][k2].x, B1[b][k2].x, B2[b][k2].x, 0.f);
            dst[2 * k + 1] = make_float4(B0[b][k2].y, B1[b][k2].y, B2[b][k2].y, 0.f);
        }
}

// Four-step shape (N1, N2, T) of the register passes for a line length; 0 when
// the length has no register pass (the shared-memory passes are used).
struct RegShape {
    int n1, n2, t;
};
static RegShape reg_shape(int N, bool z)
{
    switch (N) {
        case 4: return {4, 1, 1};
        case 8: return {4, 2, 2};
        case 16: return {4, 4, 4};
        case 32: return {8, 4, 4};
        case 64: return {8, 8, 8};
        case 128: return RegShape{16, 8, 8};
        case 256: return z ? RegShape{0, 0, 0} : RegShape{16, 16, 16};
        default: return {0, 0, 0};
    }
}

template <int N1, int N2, int T>
static void launch_y_reg(float2* spec, int nvol, int Mx, int Mzh, const float2* tw, bool inverse, const PbInst* inst,
                         const int* bucket, cudaStream_t s)
{
    const size_t sm = (size_t)N1 * N2 * 32 * sizeof(float2);
    const long long nb = (long long)nvol * Mx * ((Mzh - 1 + 31) / 32);
    if (inverse) {
        cudaFuncSetAttribute(k_fft_y_reg<N1, N2, T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_fft_y_reg<N1, N2, T, true><<<(unsigned)nb, 32 * T, sm, s>>>(spec, Mx, Mzh, tw, inst, bucket);
    } else {
        cudaFuncSetAttribute(k_fft_y_reg<N1, N2, T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_fft_y_reg<N1, N2, T, false><<<(unsigned)nb, 32 * T, sm, s>>>(spec, Mx, Mzh, tw, inst, bucket);
    }
}

template <int N1, int N2, int T>
static void launch_x_reg(float2* spec, int nb, int My, int Mzh, int Mz, long long base_off, const float2* tw,
                         const PbInst* inst, const int* bucket, cudaStream_t s)
{
    const size_t sm = (size_t)3 * N1 * N2 * 32 * sizeof(float2);
    cudaFuncSetAttribute(k_fft_x_green_reg<N1, N2, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    const long long nblk = (long long)nb * My * ((Mzh - 1 + 31) / 32);
    k_fft_x_green_reg<N1, N2, T><<<(unsigned)nblk, 32 * T, sm, s>>>(spec, inst, bucket, base_off, My, Mzh, Mz, tw);
}

template <int N1, int N2, int T>
static void launch_z_reg(const float4* grid_in, float4* grid_out, float2* spec, bool inverse, long long nlines,
                         int Mx, int My, const float2* tw, const float2* rt, const PbInst* inst, const int* bucket,
                         cudaStream_t s)
{
    constexpr int LPC = 256 / T;
    const size_t sm = (size_t)3 * N1 * N2 * LPC * sizeof(float2);
    const unsigned nblk = (unsigned)((nlines + LPC - 1) / LPC);
    if (inverse) {
        cudaFuncSetAttribute(k_fft_z_inv_reg<N1, N2, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_fft_z_inv_reg<N1, N2, T><<<nblk, 256, sm, s>>>(spec, grid_out, nlines, Mx, My, tw, rt, inst, bucket);
    } else {
        cudaFuncSetAttribute(k_fft_z_fwd_reg<N1, N2, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_fft_z_fwd_reg<N1, N2, T><<<nblk, 256, sm, s>>>(grid_in, spec, nlines, Mx, My, tw, rt, inst, bucket);
    }
}

#define PB_REG_SHAPES(X) X(4, 1, 1) X(4, 2, 2) X(4, 4, 4) X(8, 4, 4) X(8, 8, 8) X(16, 8, 8) X(16, 16, 16)
#define PB_REG_SHAPES_Z(X) X(4, 1, 1) X(4, 2, 2) X(4, 4, 4) X(8, 4, 4) X(8, 8, 8) X(16, 8, 8)

static void y_reg(RegShape r, float2* spec, int nvol, int Mx, int Mzh, const float2* tw, bool inverse,
                  const PbInst* inst, const int* bucket, cudaStream_t s)
{
#define PB_Y(a, b, c) \
    if (r.n1 == a && r.n2 == b && r.t == c) return launch_y_reg<a, b, c>(spec, nvol, Mx, Mzh, tw, inverse, inst, bucket, s);
    PB_REG_SHAPES(PB_Y)
#undef PB_Y
}

static void x_reg(RegShape r, float2* spec, int nb, int My, int Mzh, int Mz, long long base_off, const float2* tw,
                  const PbInst* inst, const int* bucket, cudaStream_t s)
{
#define PB_X(a, b, c) \
    if (r.n1 == a && r.n2 == b && r.t == c) return launch_x_reg<a, b, c>(spec, nb, My, Mzh, Mz, base_off, tw, inst, bucket, s);
    PB_REG_SHAPES(PB_X)
#undef PB_X
}

static void z_reg(RegShape r, const float4* gin, float4* gout, float2* spec, bool inverse, long long nlines, int Mx,
                  int My, const float2* tw, const float2* rt, const PbInst* inst, const int* bucket, cudaStream_t s)
{
#define PB_Z(a, b, c) \
    if (r.n1 == a && r.n2 == b && r.t == c) \
        return launch_z_reg<a, b, c>(gin, gout, spec, inverse, nlines, Mx, My, tw, rt, inst, bucket, s);
    PB_REG_SHAPES_Z(PB_Z)
#undef PB_Z
}

static int pick_tw(int N, int mult, size_t csize, int maxbytes)
{
    int tw = 16;
    while (tw > 1 && (size_t)2 * mult * tw * N * csize > (size_t)maxbytes) tw >>= 1;
    return tw;
}

template <class T>
void launch_kspace_fft(const PbInst* inst_dev, const int* bucket_inst, int nb, long long base_off, const int* M,
                       T* grid, void* spec_v, const void* tw_v, cudaStream_t s)
{
    typedef typename Cx<T>::t T2;
    T2* spec = (T2*)spec_v;
    const T2* tw = (const T2*)tw_v;
    const int Mx = M[0], My = M[1], Mz = M[2], Nh = Mz / 2, Mzh = Nh + 1;
    const int nvol = 3 * nb;
    TwOff o = tw_offsets(M);
    if (sizeof(T) == 4) {  // register passes where every axis has one
        const RegShape rz = reg_shape(Nh, true), ry = reg_shape(My, false), rx = reg_shape(Mx, false);
        if (rz.n1 && ry.n1 && rx.n1) {
            const float2* tw2 = (const float2*)tw_v;
            float2* sp2 = (float2*)spec_v;
            float4* g4 = (float4*)grid;
            const long long nlines4 = (long long)nb * Mx * My;
            z_reg(rz, g4, nullptr, sp2, false, nlines4, Mx, My, tw2 + o.zh, tw2 + o.r, inst_dev, bucket_inst, s);
            y_reg(ry, sp2, nvol, Mx, Mzh, tw2 + o.y, false, inst_dev, bucket_inst, s);
            x_reg(rx, sp2, nb, My, Mzh, Mz, base_off, tw2 + o.x, inst_dev, bucket_inst, s);
            y_reg(ry, sp2, nvol, Mx, Mzh, tw2 + o.y, true, inst_dev, bucket_inst, s);
            z_reg(rz, nullptr, g4, sp2, true, nlines4, Mx, My, tw2 + o.zh, tw2 + o.r, inst_dev, bucket_inst, s);
            return;
        }
    }
    const size_t cs = sizeof(T2);
    const int smax = 64 * 1024;
    // z forward
    long long nlines = (long long)nvol * Mx * My;
    int lpb = (int)(2048 / (Nh > 0 ? Nh : 1));
    if (lpb < 1) lpb = 1;
    size_t sm = (size_t)2 * lpb * Nh * cs;
    // FP32: interleaved float4 grid lines, three components per line
    long long nlines4 = (long long)nb * Mx * My;
    int lpb4 = std::max(1, lpb / 3);
    size_t sm4 = (size_t)2 * 3 * lpb4 * Nh * cs;
    if (sizeof(T) == 4) {
        cudaFuncSetAttribute(k_fft_z_fwd4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm4);
        k_fft_z_fwd4<<<(unsigned)((nlines4 + lpb4 - 1) / lpb4), 256, sm4, s>>>(
            (const float4*)grid, (float2*)spec, nlines4, Mx, My, Mz, lpb4, (const float2*)tw, o, inst_dev, bucket_inst);
    } else {
        cudaFuncSetAttribute(k_fft_z_fwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_fft_z_fwd<T><<<(unsigned)((nlines + lpb - 1) / lpb), 256, sm, s>>>(grid, spec, nlines, Mz, lpb, tw, o,
                                                                              (long long)Mx * My, inst_dev,
                                                                              bucket_inst);
    }
    // y forward
    int twy = pick_tw(My, 1, cs, smax);
    size_t smy = (size_t)2 * twy * My * cs;
    cudaFuncSetAttribute(k_fft_y<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smy);
    long long nby = (long long)nvol * Mx * ((Mzh + twy - 1) / twy);
    k_fft_y<T><<<(unsigned)nby, 256, smy, s>>>(spec, nvol, Mx, My, Mzh, twy, tw, o.y, false, inst_dev, bucket_inst);
    // x forward + Green + x inverse
    int twx = pick_tw(Mx, 3, cs, smax);
    size_t smx = (size_t)2 * 3 * twx * Mx * cs;
    cudaFuncSetAttribute(k_fft_x_green<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smx);
    long long nbx = (long long)nb * My * ((Mzh + twx - 1) / twx);
    k_fft_x_green<T><<<(unsigned)nbx, 256, smx, s>>>(spec, inst_dev, bucket_inst, base_off, Mx, My, Mzh, Mz, twx, tw,
                                                       o.x);
    // y inverse
    k_fft_y<T><<<(unsigned)nby, 256, smy, s>>>(spec, nvol, Mx, My, Mzh, twy, tw, o.y, true, inst_dev, bucket_inst);
    // z inverse
    if (sizeof(T) == 4) {
        cudaFuncSetAttribute(k_fft_z_inv4, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm4);
        k_fft_z_inv4<<<(unsigned)((nlines4 + lpb4 - 1) / lpb4), 256, sm4, s>>>(
            (const float2*)spec, (float4*)grid, nlines4, Mx, My, Mz, lpb4, (const float2*)tw, o, inst_dev, bucket_inst);
    } else {
        cudaFuncSetAttribute(k_fft_z_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        k_fft_z_inv<T><<<(unsigned)((nlines + lpb - 1) / lpb), 256, sm, s>>>(spec, grid, nlines, Mz, lpb, tw, o,
                                                                              (long long)Mx * My, inst_dev,
                                                                              bucket_inst);
    }
}

template void launch_kspace_fft<float>(const PbInst*, const int*, int, long long, const int*, float*, void*,
                                       const void*, cudaStream_t);
template void launch_kspace_fft<double>(const PbInst*, const int*, int, long long, const int*, double*, void*,
                                        const void*, cudaStream_t);

// ---------------------------------------------------------------------------
// Final FP64 combine and force sums
// ---------------------------------------------------------------------------
__global__ void k_combine_mixed(const PbInst* __restrict__ inst, int ninst, const int* __restrict__ tgt_offsets,
                                const int* __restrict__ tperm, const double* __restrict__ u_real,
                                const float* __restrict__ u_k, int use_real, int use_k, const double* __restrict__ fsum,
                                const PbTables* __restrict__ tab, const double* __restrict__ frc,
                                const int* __restrict__ src_offsets, double* __restrict__ U)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tgt_offsets[ninst]) return;
    int p = tperm[t];
    int q = find_instance(tgt_offsets, ninst, p);
    const PbInst& I = inst[q];
    double tau = I.L[0] * I.L[1] * I.L[2];
    // self pair (targets are the sources): (R_eps(0) - R_d(0)) f_i in FP64
    const bool self = use_real && I.same && (I.flags & 1);
    const size_t ps = (size_t)(p - tgt_offsets[q] + src_offsets[q]);
    for (int c = 0; c < 3; c++) {
        double v = 0;
        size_t o = 3 * (size_t)t + c;
        if (self) v += tab[q].self1 * frc[3 * ps + c];
        if (use_real && (I.flags & 1)) v += u_real[o];
        if (use_k && (I.flags & 2)) v += (double)u_k[o];
        if (I.flags & 4) v += fsum[3 * q + c] / (I.alpha * I.alpha * tau);
        U[3 * (size_t)p + c] = v;
    }
}

__global__ void k_combine_fp64(const PbInst* __restrict__ inst, int ninst, const int* __restrict__ tgt_offsets,
                               const int* __restrict__ tperm, const double* __restrict__ u_real,
                               const double* __restrict__ u_k, int use_real, int use_k,
                               const double* __restrict__ fsum, const PbTables* __restrict__ tab,
                               const double* __restrict__ frc, const int* __restrict__ src_offsets,
                               double* __restrict__ U)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= tgt_offsets[ninst]) return;
    int p = tperm[t];
    int q = find_instance(tgt_offsets, ninst, p);
    const PbInst& I = inst[q];
    double tau = I.L[0] * I.L[1] * I.L[2];
    const bool self = use_real && I.same && (I.flags & 1);
    const size_t ps = (size_t)(p - tgt_offsets[q] + src_offsets[q]);
    for (int c = 0; c < 3; c++) {
        double v = 0;
        size_t o = 3 * (size_t)t + c;
        if (self) v += tab[q].self1 * frc[3 * ps + c];
        if (use_real && (I.flags & 1)) v += u_real[o];
        if (use_k && (I.flags & 2)) v += u_k[o];
        if (I.flags & 4) v += fsum[3 * q + c] / (I.alpha * I.alpha * tau);
        U[3 * (size_t)p + c] = v;
    }
}

void launch_combine_mixed(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const int* tperm,
                          const double* u_real, const float* u_k, int use_real, int use_k, const double* fsum,
                          const PbTables* tab, const double* frc, const int* src_offsets, double* U, cudaStream_t s)
{
    if (ncap <= 0) return;
    k_combine_mixed<<<(ncap + 255) / 256, 256, 0, s>>>(inst, ninst, tgt_offsets, tperm, u_real, u_k, use_real, use_k,
                                                        fsum, tab, frc, src_offsets, U);
}

void launch_combine_fp64(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const int* tperm,
                         const double* u_real, const double* u_k, int use_real, int use_k, const double* fsum,
                         const PbTables* tab, const double* frc, const int* src_offsets, double* U, cudaStream_t s)
{
    if (ncap <= 0) return;
    k_combine_fp64<<<(ncap + 255) / 256, 256, 0, s>>>(inst, ninst, tgt_offsets, tperm, u_real, u_k, use_real,
                                                       use_k, fsum, tab, frc, src_offsets, U);
}

// Per-instance force sums for the k = 0 mode (only instances that ask for it):
// blockIdx.y = instance, blocks stride over its sources, FP64 atomics.
__global__ void k_force_sums(const PbInst* __restrict__ inst, const double* __restrict__ frc,
                             const int* __restrict__ offsets, double* __restrict__ out)
{
    const int q = blockIdx.y;
    if (!(inst[q].flags & 4)) return;
    const int b = offsets[q], e = offsets[q + 1];
    double s[3] = {0, 0, 0};
    for (int p = b + blockIdx.x * blockDim.x + threadIdx.x; p < e; p += gridDim.x * blockDim.x)
        for (int c = 0; c < 3; c++) s[c] += frc[3 * (size_t)p + c];
#pragma unroll
    for (int c = 0; c < 3; c++)
        for (int o = 16; o > 0; o >>= 1) s[c] += __shfl_xor_sync(kFull, s[c], o);
    if ((threadIdx.x & 31) == 0)
        for (int c = 0; c < 3; c++) atomicAdd(&out[3 * q + c], s[c]);
}

void launch_force_sums(const PbInst* inst, const double* frc, const int* offsets, int ninst, double* out,
                       cudaStream_t s)
{
    if (ninst <= 0) return;
    cudaMemsetAsync(out, 0, 3 * sizeof(double) * (size_t)ninst, s);
    k_force_sums<<<dim3(16, (unsigned)ninst), 256, 0, s>>>(inst, frc, offsets, out);
}

}  // namespace pb
