// Real-space Ewald sum over a device-built cell list.
//
// Work item = (instance, target cell, chunk of <= 32 targets), one warp per
// item, items pulled from a global counter by a persistent grid.  Each lane
// owns one target.  The sources of the (2S+1)^3 stencil are visited as
// contiguous z-runs of the cell-sorted source array, staged 32 at a time in
// shared memory; a first pass builds a per-lane bit mask of the sources inside
// the cutoff, a second pass evaluates only those pairs.
//
// Mixed precision (k_real_mixed): positions are FP32 hi/lo pairs re-expressed
// in the frame of the target cell (error-free TwoSum), so displacements carry
// FP32 relative accuracy even at r << cell size; the pair kernel is the FP32
// polynomial T(r) of the instance tables (FMA only); per-chunk partial sums are
// Kahan-accumulated; pairs below r_tiny use the FP64 series and an FP64
// accumulator.  The self pair of targets that are the sources is skipped here
// and added in FP64 by the combine kernel (R_eps(0) - R_d(0)) f_i.
//
// FP64 (k_real_fp64): the reference's closed forms (cuda/periodicBrinkman.h:85-176)
// in double precision, FP64 series below r_tiny.
#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

constexpr int kRealWarps = 4;

struct ItemFrame {
    int q, c0, c1, c2;
    double O[3];
};

__device__ __forceinline__ void item_frame(const PbInst& I, int4 it, ItemFrame& F)
{
    int local = it.y - I.cell_off;
    F.q = it.x;
    F.c2 = local % I.nc[2];
    int r = local / I.nc[2];
    F.c1 = r % I.nc[1];
    F.c0 = r / I.nc[1];
    F.O[0] = F.c0 * I.h[0];
    F.O[1] = F.c1 * I.h[1];
    F.O[2] = F.c2 * I.h[2];
}

template <int NP>
__device__ __forceinline__ float horner(const float (&c)[NP], float t)
{
    float h = c[NP - 1];
#pragma unroll
    for (int k = NP - 2; k >= 0; k--) h = fmaf(h, t, c[k]);
    return h;
}

__device__ __forceinline__ float horner_g(const float* __restrict__ c, int n, float t)
{
    float h = __ldg(&c[n - 1]);
    for (int k = n - 2; k >= 0; k--) h = fmaf(h, t, __ldg(&c[k]));
    return h;
}

template <int NP>
__global__ void __launch_bounds__(kRealWarps * 32)
    k_real_mixed(const PbInst* __restrict__ inst, const PbTables* __restrict__ tab, const int4* __restrict__ items,
                 const int* __restrict__ nitems_ptr, const float4* __restrict__ spos_hi, const float4* __restrict__ spos_lo,
                 const float4* __restrict__ sfrc, const int* __restrict__ src_start, const float4* __restrict__ tpos_hi,
                 const float4* __restrict__ tpos_lo, float* __restrict__ u_s, float* __restrict__ u_c,
                 double* __restrict__ u_near, int* __restrict__ counter)
{
    __shared__ float4 sh_hi[kRealWarps][32];
    __shared__ float4 sh_lo[kRealWarps][32];
    __shared__ float4 sh_f[kRealWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;

    const int nitems = *nitems_ptr;
    float c1[NP], c2[NP];
    int cur_q = -1;
    float tds = 0, tdo = 0, rc2 = 0, rs2 = 0, rtiny2 = 0, tes = 0, teo = 0;
    int ne = 0;

    while (true) {
        int item = 0;
        if (lane == 0) item = atomicAdd(counter, 1);
        item = __shfl_sync(kFull, item, 0);
        if (item >= nitems) break;
        const int4 it = items[item];
        const PbInst& I = inst[it.x];
        const PbTables& T = tab[it.x];
        if (it.x != cur_q) {
            cur_q = it.x;
#pragma unroll
            for (int k = 0; k < NP; k++) {
                c1[k] = T.pd1[k];
                c2[k] = T.pd2[k];
            }
            tds = T.td_scale;
            tdo = T.td_off;
            rc2 = T.rc2;
            rs2 = T.rs2;
            rtiny2 = T.rtiny2f;
            tes = T.te_scale;
            teo = T.te_off;
            ne = T.ne;
        }
        ItemFrame F;
        item_frame(I, it, F);
        const bool active = lane < it.w;
        const int tidx = it.z + (active ? lane : 0);
        // sorted index of this target among the sources when targets are the sources
        const int self_src = I.same ? tidx - I.tgt_off + I.src_off : -1;
        // target in the cell frame, hi + lo
        float th[3], tl[3];
        {
            float4 ph = tpos_hi[tidx], pl = tpos_lo[tidx];
            float xh[3] = {ph.x, ph.y, ph.z}, xl[3] = {pl.x, pl.y, pl.z};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                float oh, ol, s, e;
                split_double(F.O[a], oh, ol);
                two_sum(xh[a], -oh, s, e);
                th[a] = s;
                tl[a] = e + (xl[a] - ol);
            }
        }
        float s0 = 0, s1 = 0, s2 = 0, k0 = 0, k1 = 0, k2 = 0;
        double n0 = 0, n1 = 0, n2 = 0;

        for (int o0 = -I.S[0]; o0 <= I.S[0]; o0++) {
            int g0 = F.c0 + o0;
            int w0 = ((g0 % I.nc[0]) + I.nc[0]) % I.nc[0];
            double sh0 = (double)((g0 - w0) / I.nc[0]) * I.L[0];
            for (int o1 = -I.S[1]; o1 <= I.S[1]; o1++) {
                int g1 = F.c1 + o1;
                int w1 = ((g1 % I.nc[1]) + I.nc[1]) % I.nc[1];
                double sh1 = (double)((g1 - w1) / I.nc[1]) * I.L[1];
                int row = I.cell_off + (w0 * I.nc[1] + w1) * I.nc[2];
                int g2 = F.c2 - I.S[2];
                const int g2end = F.c2 + I.S[2];
                while (g2 <= g2end) {
                    // maximal run of unwrapped z cells sharing one image shift
                    int w2 = ((g2 % I.nc[2]) + I.nc[2]) % I.nc[2];
                    int run = min(g2end - g2 + 1, I.nc[2] - w2);
                    double sh2 = (double)((g2 - w2) / I.nc[2]) * I.L[2];
                    int b = src_start[row + w2], e = src_start[row + w2 + run];
                    g2 += run;
                    const bool zero_shift = (sh0 == 0.0) && (sh1 == 0.0) && (sh2 == 0.0);
                    float qh[3], ql[3];
                    split_double(F.O[0] - sh0, qh[0], ql[0]);
                    split_double(F.O[1] - sh1, qh[1], ql[1]);
                    split_double(F.O[2] - sh2, qh[2], ql[2]);
                    for (int base = b; base < e; base += 32) {
                        int j = base + lane;
                        if (j < e) {
                            float4 ph = spos_hi[j], pl = spos_lo[j];
                            float xh[3] = {ph.x, ph.y, ph.z}, xl[3] = {pl.x, pl.y, pl.z};
                            float ph3[3], pl3[3];
#pragma unroll
                            for (int a = 0; a < 3; a++) {
                                float s, er;
                                two_sum(xh[a], -qh[a], s, er);
                                ph3[a] = s;
                                pl3[a] = er + (xl[a] - ql[a]);
                            }
                            sh_hi[w][lane] = make_float4(ph3[0], ph3[1], ph3[2], 0.f);
                            sh_lo[w][lane] = make_float4(pl3[0], pl3[1], pl3[2], 0.f);
                            sh_f[w][lane] = sfrc[j];
                        }
                        __syncwarp();
                        const int ncand = min(32, e - base);
                        unsigned mask = 0;
                        if (active) {
                            for (int jj = 0; jj < ncand; jj++) {
                                float4 p = sh_hi[w][jj];
                                float dx = th[0] - p.x, dy = th[1] - p.y, dz = th[2] - p.z;
                                float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                mask |= (r2 < rc2 ? 1u : 0u) << jj;
                            }
                            // the self pair (targets are the sources, same particle, no shift)
                            // is added in FP64 by the combine kernel
                            if (self_src >= base && self_src < base + ncand && zero_shift)
                                mask &= ~(1u << (self_src - base));
                        }
                        float a0 = 0, a1 = 0, a2 = 0;
                        while (__any_sync(kFull, mask)) {
                            if (mask) {
                                int jj = __ffs(mask) - 1;
                                mask &= mask - 1;
                                float4 p = sh_hi[w][jj], pl = sh_lo[w][jj], f = sh_f[w][jj];
                                float dx = (th[0] - p.x) + (tl[0] - pl.x);
                                float dy = (th[1] - p.y) + (tl[1] - pl.y);
                                float dz = (th[2] - p.z) + (tl[2] - pl.z);
                                float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                if (r2 < rtiny2 || r2 == 0.f) {
                                    double H1, H2;
                                    double ddx = dx, ddy = dy, ddz = dz;
                                    double rr = ddx * ddx + ddy * ddy + ddz * ddz;
                                    if (T.blob) {
                                        series_H(T, rr, H1, H2);
                                    } else {
                                        H1 = T.self1;
                                        H2 = 0;
                                    }
                                    double fd = f.x * ddx + f.y * ddy + f.z * ddz;
                                    n0 += H1 * f.x + H2 * fd * ddx;
                                    n1 += H1 * f.y + H2 * fd * ddy;
                                    n2 += H1 * f.z + H2 * fd * ddz;
                                } else {
                                    float ri = rsqrtf(r2);
                                    ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);
                                    float r = r2 * ri;
                                    float t = fmaf(r, tds, tdo);
                                    float T1 = horner<NP>(c1, t);
                                    float T2 = horner<NP>(c2, t);
                                    if (r2 < rs2) {
                                        float te = fmaf(r, tes, teo);
                                        T1 -= horner_g(T.pe1, ne, te);
                                        T2 -= horner_g(T.pe2, ne, te);
                                    }
                                    float H1 = T1 * ri;
                                    float H2 = T2 * (ri * ri * ri);
                                    float fd = fmaf(f.x, dx, fmaf(f.y, dy, f.z * dz));
                                    float g = H2 * fd;
                                    a0 = fmaf(H1, f.x, fmaf(g, dx, a0));
                                    a1 = fmaf(H1, f.y, fmaf(g, dy, a1));
                                    a2 = fmaf(H1, f.z, fmaf(g, dz, a2));
                                }
                            }
                        }
                        kahan_add(s0, k0, a0);
                        kahan_add(s1, k1, a1);
                        kahan_add(s2, k2, a2);
                        __syncwarp();
                    }
                }
            }
        }
        if (active) {
            size_t o = 3 * (size_t)tidx;
            u_s[o] = s0;
            u_s[o + 1] = s1;
            u_s[o + 2] = s2;
            u_c[o] = k0;
            u_c[o + 1] = k1;
            u_c[o + 2] = k2;
            u_near[o] = n0;
            u_near[o + 1] = n1;
            u_near[o + 2] = n2;
        }
    }
}

void launch_real_mixed(int npoly, const PbInst* inst, const PbTables* tab, const int4* items, const int* nitems_ptr,
                       int nitems_max,
                       const float4* spos_hi, const float4* spos_lo, const float4* sfrc, const int* src_start,
                       const float4* tpos_hi, const float4* tpos_lo, float* u_s, float* u_c, double* u_near,
                       int* counter, int nsm, cudaStream_t s)
{
    if (nitems_max <= 0) return;
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    int blocks = nsm * 8;
    int need = (nitems_max + kRealWarps - 1) / kRealWarps;
    if (blocks > need) blocks = need;
#define PB_LAUNCH_REAL(NP)                                                                                            \
    k_real_mixed<NP><<<blocks, kRealWarps * 32, 0, s>>>(inst, tab, items, nitems_ptr, spos_hi, spos_lo, sfrc,        \
                                                         src_start,                                                  \
                                                         tpos_hi, tpos_lo, u_s, u_c, u_near, counter)
    if (npoly <= 16)
        PB_LAUNCH_REAL(16);
    else if (npoly <= 20)
        PB_LAUNCH_REAL(20);
    else if (npoly <= 24)
        PB_LAUNCH_REAL(24);
    else
        PB_LAUNCH_REAL(28);
#undef PB_LAUNCH_REAL
}

__global__ void __launch_bounds__(kRealWarps * 32)
    k_real_fp64(const PbInst* __restrict__ inst, const PbTables* __restrict__ tab, const int4* __restrict__ items,
                const int* __restrict__ nitems_ptr, const Dbl4* __restrict__ spos, const Dbl4* __restrict__ sfrc,
                const int* __restrict__ src_start, const Dbl4* __restrict__ tpos, double* __restrict__ u,
                int* __restrict__ counter)
{
    __shared__ Dbl4 sh_p[kRealWarps][32];
    __shared__ Dbl4 sh_f[kRealWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nitems = *nitems_ptr;
    while (true) {
        int item = 0;
        if (lane == 0) item = atomicAdd(counter, 1);
        item = __shfl_sync(kFull, item, 0);
        if (item >= nitems) break;
        const int4 it = items[item];
        const PbInst& I = inst[it.x];
        const PbTables& T = tab[it.x];
        const double a = I.alpha, dd = I.d, ee = I.eps;
        const double cd = -expm1(-a * a * dd * dd / 4), ce = -expm1(-a * a * ee * ee / 4);
        const double rc2 = I.rc * I.rc;
        const double rs2 = (double)T.rs2;
        ItemFrame F;
        item_frame(I, it, F);
        const bool active = lane < it.w;
        const int tidx = it.z + (active ? lane : 0);
        const int self_src = I.same ? tidx - I.tgt_off + I.src_off : -1;
        Dbl4 tp = tpos[tidx];
        double v0 = 0, v1 = 0, v2 = 0;
        for (int o0 = -I.S[0]; o0 <= I.S[0]; o0++) {
            int g0 = F.c0 + o0;
            int w0 = ((g0 % I.nc[0]) + I.nc[0]) % I.nc[0];
            double sh0 = (double)((g0 - w0) / I.nc[0]) * I.L[0];
            for (int o1 = -I.S[1]; o1 <= I.S[1]; o1++) {
                int g1 = F.c1 + o1;
                int w1 = ((g1 % I.nc[1]) + I.nc[1]) % I.nc[1];
                double sh1 = (double)((g1 - w1) / I.nc[1]) * I.L[1];
                int row = I.cell_off + (w0 * I.nc[1] + w1) * I.nc[2];
                int g2 = F.c2 - I.S[2];
                const int g2end = F.c2 + I.S[2];
                while (g2 <= g2end) {
                    int w2 = ((g2 % I.nc[2]) + I.nc[2]) % I.nc[2];
                    int run = min(g2end - g2 + 1, I.nc[2] - w2);
                    double sh2 = (double)((g2 - w2) / I.nc[2]) * I.L[2];
                    int b = src_start[row + w2], e = src_start[row + w2 + run];
                    g2 += run;
                    const bool zero_shift = (sh0 == 0.0) && (sh1 == 0.0) && (sh2 == 0.0);
                    for (int base = b; base < e; base += 32) {
                        int j = base + lane;
                        if (j < e) {
                            Dbl4 p = spos[j];
                            sh_p[w][lane] = make_dbl4(p.x + sh0, p.y + sh1, p.z + sh2, 0.0);
                            sh_f[w][lane] = sfrc[j];
                        }
                        __syncwarp();
                        const int ncand = min(32, e - base);
                        unsigned mask = 0;
                        if (active) {
                            for (int jj = 0; jj < ncand; jj++) {
                                Dbl4 p = sh_p[w][jj];
                                double dx = tp.x - p.x, dy = tp.y - p.y, dz = tp.z - p.z;
                                double r2 = dx * dx + dy * dy + dz * dz;
                                mask |= (r2 < rc2 ? 1u : 0u) << jj;
                            }
                            if (self_src >= base && self_src < base + ncand && zero_shift)
                                mask &= ~(1u << (self_src - base));
                        }
                        while (__any_sync(kFull, mask)) {
                            if (mask) {
                                int jj = __ffs(mask) - 1;
                                mask &= mask - 1;
                                Dbl4 p = sh_p[w][jj], f = sh_f[w][jj];
                                double dx = tp.x - p.x, dy = tp.y - p.y, dz = tp.z - p.z;
                                double r2 = dx * dx + dy * dy + dz * dz;
                                double H1, H2;
                                if (r2 < T.rtiny2 || r2 == 0.0) {
                                    if (T.blob) {
                                        series_H(T, r2, H1, H2);
                                    } else {
                                        H1 = T.self1;
                                        H2 = 0;
                                    }
                                } else {
                                    double r = sqrt(r2);
                                    diffH_d(r, a, dd, cd, H1, H2);
                                    if (T.blob && r2 < rs2) {
                                        double e1, e2;
                                        diffH_d(r, a, ee, ce, e1, e2);
                                        H1 -= e1;
                                        H2 -= e2;
                                    }
                                }
                                double fd = f.x * dx + f.y * dy + f.z * dz;
                                v0 += H1 * f.x + H2 * fd * dx;
                                v1 += H1 * f.y + H2 * fd * dy;
                                v2 += H1 * f.z + H2 * fd * dz;
                            }
                        }
                        __syncwarp();
                    }
                }
            }
        }
        if (active) {
            size_t o = 3 * (size_t)tidx;
            u[o] = v0;
            u[o + 1] = v1;
            u[o + 2] = v2;
        }
    }
}

void launch_real_fp64(const PbInst* inst, const PbTables* tab, const int4* items, const int* nitems_ptr,
                      int nitems_max, const Dbl4* spos, const Dbl4* sfrc, const int* src_start,
                      const Dbl4* tpos, double* u, int* counter, int nsm, cudaStream_t s)
{
    if (nitems_max <= 0) return;
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    int blocks = nsm * 8;
    int need = (nitems_max + kRealWarps - 1) / kRealWarps;
    if (blocks > need) blocks = need;
    k_real_fp64<<<blocks, kRealWarps * 32, 0, s>>>(inst, tab, items, nitems_ptr, spos, sfrc, src_start, tpos, u,
                                                   counter);
}

}  // namespace pb
