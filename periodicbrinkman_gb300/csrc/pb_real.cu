// Real-space Ewald sum over a device-built cell list.
//
// Work item = (instance, cell row (c0, c1), z-range [za, zb] of at most 8
// cells, up to 32 consecutive sorted targets), one warp per item, items pulled
// from a global counter by a persistent grid.  Each lane owns one target.  The
// sources of the stencil (rows c0 +- S, c1 +- S; cells za - S .. zb + S) are
// visited as contiguous z-runs of the cell-sorted source array, staged 32 at a
// time in shared memory.  Mixed precision: each lane classifies its 32 candidate
// pairs (inside the cutoff / inside the blob region / below r_tiny), the warp
// compacts them into target-major queues in shared memory, and every lane then
// evaluates one queued pair at a time, so the FMA pipe sees full warps and the
// rare blob and series pairs never diverge the common path; per-target sums
// of each round are formed by a segmented warp reduction (no atomics).
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

constexpr int kMaxReach = 15;  // stencil reach S per axis
constexpr int kZTab = 8 + 2 * kMaxReach;

// item = {instance, first target, local row c0*nc1 + c1, count | za << 8 | zb << 16 | group << 24}:
// the item covers the stencil columns col = group, group + csplit, ... of its rows
struct ItemFrame {
    int q, c0, c1, za, zb, first, count, group;
    double O[3];
};

__device__ __forceinline__ void item_frame(const PbInst& I, int4 it, ItemFrame& F)
{
    F.q = it.x;
    F.first = it.y;
    F.c0 = it.z / I.nc[1];
    F.c1 = it.z % I.nc[1];
    F.count = it.w & 0xff;
    F.za = (it.w >> 8) & 0xff;
    F.zb = (it.w >> 16) & 0xff;
    F.group = (it.w >> 24) & 0xff;
    F.O[0] = F.c0 * I.h[0];
    F.O[1] = F.c1 * I.h[1];
    F.O[2] = F.za * I.h[2];
}

// Per-item frame tables: for every stencil offset along an axis, the wrapped
// cell index, whether the image shift is zero, and Q = O - shift as an FP32
// hi/lo pair, so the inner loops need no FP64.
struct __align__(8) FrameTabs {
    float2 qx[2 * kMaxReach + 1], qy[2 * kMaxReach + 1], qz[kZTab];
    int wx[2 * kMaxReach + 1], wy[2 * kMaxReach + 1], wz[kZTab];
    int zx[2 * kMaxReach + 1], zy[2 * kMaxReach + 1], zz[kZTab];
};

__device__ __forceinline__ void fill_frame_tabs(const PbInst& I, const ItemFrame& F, FrameTabs& T, int lane)
{
    const int nx = 2 * I.S[0] + 1, ny = 2 * I.S[1] + 1, nz = F.zb - F.za + 2 * I.S[2] + 1;
    for (int i = lane; i < nx + ny + nz; i += 32) {
        int ax, g, k;
        if (i < nx) {
            ax = 0;
            k = i;
            g = F.c0 + i - I.S[0];
        } else if (i < nx + ny) {
            ax = 1;
            k = i - nx;
            g = F.c1 + k - I.S[1];
        } else {
            ax = 2;
            k = i - nx - ny;
            g = F.za + k - I.S[2];
        }
        const int n = I.nc[ax];
        int w = ((g % n) + n) % n;
        int sc = (g - w) / n;  // image shift count
        double Q = F.O[ax] - (double)sc * I.L[ax];
        float hi, lo;
        split_double(Q, hi, lo);
        if (ax == 0) {
            T.qx[k] = make_float2(hi, lo);
            T.wx[k] = w;
            T.zx[k] = sc == 0;
        } else if (ax == 1) {
            T.qy[k] = make_float2(hi, lo);
            T.wy[k] = w;
            T.zy[k] = sc == 0;
        } else {
            T.qz[k] = make_float2(hi, lo);
            T.wz[k] = w;
            T.zz[k] = sc == 0;
        }
    }
}

// Both polynomials (T1, T2) of one argument in packed FP32x2 FMAs.
template <int NP>
__device__ __forceinline__ float2 horner2(const float2 (&c)[NP], float t)
{
    const float2 tt = make_float2(t, t);
    float2 h = c[NP - 1];
#pragma unroll
    for (int k = NP - 2; k >= 0; k--) h = __ffma2_rn(h, tt, c[k]);
    return h;
}

// Chebyshev series (two at once) by the Clenshaw recurrence; coefficients in
// shared memory, the same for the whole warp.
__device__ __forceinline__ float2 cheb2(const float2* __restrict__ c, int n, float t)
{
    const float2 t2 = make_float2(2.f * t, 2.f * t);
    float2 b1 = make_float2(0.f, 0.f), b2 = b1;
    for (int k = n - 1; k >= 1; k--) {
        const float2 ck = c[k];
        const float2 b0 = __ffma2_rn(t2, b1, make_float2(ck.x - b2.x, ck.y - b2.y));
        b2 = b1;
        b1 = b0;
    }
    const float2 c0 = c[0];
    return __ffma2_rn(make_float2(t, t), b1, make_float2(c0.x - b2.x, c0.y - b2.y));
}

__device__ __forceinline__ float horner_g(const float* __restrict__ c, int n, float t)
{
    float h = __ldg(&c[n - 1]);
    for (int k = n - 2; k >= 0; k--) h = fmaf(h, t, __ldg(&c[k]));
    return h;
}

// Per-warp shared memory of the mixed-precision kernel.
struct __align__(16) RealWarpSmem {
    float4 s_hi[32], s_lo[32], s_f[32];  // staged sources: frame-relative hi, lo; force
    float4 t_hi[32], t_lo[32];           // the item's targets: frame-relative hi, lo
    float c_x[32], c_y[32], c_z[32];     // staged sources, hi parts by axis (classification)
    float acc[3][32];                    // per-target partial sums of the current chunk
    double acc64[3][32];                 // per-target FP64 sums of series pairs
    unsigned short q[3][1024];           // pair queues (t << 5 | j): screened, blob region, series
    float2 tn[kMaxCheb];                 // near piece (T1, T2) of the current instance
    float2 tb[kMaxCheb];                 // blob piece (H1, r^2 H2) of the current instance
    FrameTabs ft;                        // the current item's frame tables
};

// Warp-wide exclusive prefix sum (64-bit, three packed 16-bit counters).
__device__ __forceinline__ unsigned long long warp_excl_scan64(unsigned long long v, int lane)
{
    unsigned long long x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    return x - v;
}

// Segmented (by target) warp reduction of the contributions of one round of
// a target-major queue; segment ends add into the per-target accumulators.
__device__ __forceinline__ void segment_reduce_add(float v0, float v1, float v2, int key, int lane, float (*acc)[32])
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        float a0 = __shfl_up_sync(kFull, v0, o), a1 = __shfl_up_sync(kFull, v1, o), a2 = __shfl_up_sync(kFull, v2, o);
        int kk = __shfl_up_sync(kFull, key, o);
        if (lane >= o && kk == key) {
            v0 += a0;
            v1 += a1;
            v2 += a2;
        }
    }
    int knext = __shfl_down_sync(kFull, key, 1);
    if (key >= 0 && (lane == 31 || knext != key)) {
        acc[0][key] += v0;
        acc[1][key] += v1;
        acc[2][key] += v2;
    }
}

template <int NP>
__global__ void __launch_bounds__(kRealWarps * 32, 4)
    k_real_mixed(const PbInst* __restrict__ inst, const PbTables* __restrict__ tab, const int4* __restrict__ items,
                 const int* __restrict__ nitems_ptr, const float4* __restrict__ spos_hi, const float4* __restrict__ spos_lo,
                 const float4* __restrict__ sfrc, const int* __restrict__ src_start, const float4* __restrict__ tpos_hi,
                 const float4* __restrict__ tpos_lo, double* __restrict__ u_real, int* __restrict__ counter,
                 int item_cap)
{
    __shared__ RealWarpSmem smem_all[kRealWarps];
    RealWarpSmem& S = smem_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;

    const int nitems = min(*nitems_ptr, item_cap);
    float2 c12[NP];
    int cur_q = -1;
    float tds = 0, tdo = 0, rc2 = 0, rare2 = 0, rtiny2 = 0, tbs = 0, tbo = 0, tns = 0, tno = 0, rs2 = 0;
    int nbp = 1, nnp = 1;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        S.acc[c][lane] = 0.f;
        S.acc64[c][lane] = 0.0;
    }

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
            for (int k = 0; k < NP; k++) c12[k] = make_float2(T.pd1[k], T.pd2[k]);
            tds = T.td_scale;
            tdo = T.td_off;
            rc2 = T.rc2;
            // rare pairs: the blob region (eps > 0), else coincident points only
            rare2 = T.rm2;  // near piece (holds the blob region and r = 0)
            rs2 = T.rs2;
            tns = T.tn_scale;
            tno = T.tn_off;
            nnp = T.nn > 0 ? T.nn : 1;
            rtiny2 = T.rtiny2f;
            tbs = T.tb_scale;
            tbo = T.tb_off;
            nbp = T.nb > 0 ? T.nb : 1;
            for (int k = lane; k < kMaxCheb; k += 32) {
                S.tn[k] = make_float2(T.cn1[k], T.cn2[k]);
                S.tb[k] = make_float2(T.cb1[k], T.cb2[k]);
            }
        }
        ItemFrame F;
        item_frame(I, it, F);
        fill_frame_tabs(I, F, S.ft, lane);
        const bool active = lane < F.count;
        const int tidx = F.first + (active ? lane : 0);
        const int self_src = I.same ? tidx - I.tgt_off + I.src_off : -1;
        float th[3], tl[3];
        {
            float4 ph = tpos_hi[tidx], pl = tpos_lo[tidx];
            float xh[3] = {ph.x, ph.y, ph.z}, xl[3] = {pl.x, pl.y, pl.z};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                float oh, ol, s, e;
                split_double(F.O[a], oh, ol);
                two_sum(xh[a], -oh, s, e);
                th[a] = active ? s : 3.0e30f;  // inactive lanes pair with nothing
                tl[a] = e + (xl[a] - ol);
            }
        }
        S.t_hi[lane] = make_float4(th[0], th[1], th[2], 0.f);
        S.t_lo[lane] = make_float4(tl[0], tl[1], tl[2], 0.f);
        __syncwarp();
        float s0 = 0, s1 = 0, s2 = 0, k0 = 0, k1 = 0, k2 = 0;
        const int nzt = F.zb - F.za + 2 * I.S[2] + 1;

        const int ny1 = 2 * I.S[1] + 1, ncol = (2 * I.S[0] + 1) * ny1;
        const int csplit = max(1, I.csplit);
        for (int col = F.group; col < ncol; col += csplit) {
            const int i0 = col / ny1, i1 = col - i0 * ny1;
            {
                const float2 qx = S.ft.qx[i0];
                const int w0 = S.ft.wx[i0], z0 = S.ft.zx[i0];
                const float2 qy = S.ft.qy[i1];
                const int w1 = S.ft.wy[i1], z1 = S.ft.zy[i1];
                const int row = I.cell_off + (w0 * I.nc[1] + w1) * I.nc[2];
                int i2 = 0;
                while (i2 < nzt) {
                    // maximal run of z cells sharing one image shift (contiguous wrapped cells)
                    const int w2 = S.ft.wz[i2];
                    const int run = min(nzt - i2, I.nc[2] - w2);
                    const float2 qz = S.ft.qz[i2];
                    const bool zero_shift = z0 && z1 && S.ft.zz[i2];
                    const int b = src_start[row + w2], e = src_start[row + w2 + run];
                    i2 += run;
                    const float qh[3] = {qx.x, qy.x, qz.x}, ql[3] = {qx.y, qy.y, qz.y};
                    for (int base = b; base < e; base += 32) {
                        const int j = base + lane;
                        const int ncand = min(32, e - base);
                        if (lane < ncand) {
                            float4 ph = spos_hi[j], pl = spos_lo[j];
                            float xh[3] = {ph.x, ph.y, ph.z}, xl[3] = {pl.x, pl.y, pl.z};
                            float p3[3], l3[3];
#pragma unroll
                            for (int a = 0; a < 3; a++) {
                                float s, er;
                                two_sum(xh[a], -qh[a], s, er);
                                p3[a] = s;
                                l3[a] = er + (xl[a] - ql[a]);
                            }
                            S.s_hi[lane] = make_float4(p3[0], p3[1], p3[2], 0.f);
                            S.s_lo[lane] = make_float4(l3[0], l3[1], l3[2], 0.f);
                            S.s_f[lane] = sfrc[j];
                            S.c_x[lane] = p3[0];
                            S.c_y[lane] = p3[1];
                            S.c_z[lane] = p3[2];
                        } else {  // padding: far from every target, active (finite) or not (+3e30)
                            S.c_x[lane] = -3.0e30f;
                            S.c_y[lane] = -3.0e30f;
                            S.c_z[lane] = -3.0e30f;
                        }
                        __syncwarp();
                        // classify candidate pairs of this lane's target: screened / blob region / series
                        // (two candidates per packed FP32x2 operation; padded to 32)
                        unsigned mi = 0, mr = 0;
                        {
                            const float2 ntx = make_float2(-th[0], -th[0]), nty = make_float2(-th[1], -th[1]),
                                         ntz = make_float2(-th[2], -th[2]);
#pragma unroll
                            for (int jj = 0; jj < 32; jj += 2) {
                                const float2 dx = __fadd2_rn(*reinterpret_cast<const float2*>(&S.c_x[jj]), ntx);
                                const float2 dy = __fadd2_rn(*reinterpret_cast<const float2*>(&S.c_y[jj]), nty);
                                const float2 dz = __fadd2_rn(*reinterpret_cast<const float2*>(&S.c_z[jj]), ntz);
                                float2 r2 = __fmul2_rn(dx, dx);
                                r2 = __ffma2_rn(dy, dy, r2);
                                r2 = __ffma2_rn(dz, dz, r2);
                                if (r2.x < rc2) mi |= 1u << jj;
                                if (r2.y < rc2) mi |= 2u << jj;
                                if (r2.x < rare2) mr |= 1u << jj;
                                if (r2.y < rare2) mr |= 2u << jj;
                            }
                        }
                        unsigned mn = mi & ~mr, mb = 0, ms = 0;
                        for (unsigned m = mr; m; m &= m - 1) {  // rare: blob region or series
                            const int jj = __ffs(m) - 1;
                            float4 p = S.s_hi[jj];
                            float dx = th[0] - p.x, dy = th[1] - p.y, dz = th[2] - p.z;
                            float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                            if ((r2 < rtiny2) | (r2 == 0.f))
                                ms |= 1u << jj;
                            else
                                mb |= 1u << jj;
                        }
                        if (zero_shift && self_src >= base && self_src < base + ncand)
                            ms &= ~(1u << (self_src - base));  // self pair: added in FP64 by the combine kernel
                        // target-major queues
                        unsigned long long cnt = (unsigned long long)__popc(mn) |
                                                 ((unsigned long long)__popc(mb) << 16) |
                                                 ((unsigned long long)__popc(ms) << 32);
                        unsigned long long ex = warp_excl_scan64(cnt, lane);
                        unsigned long long tot = __shfl_sync(kFull, ex + cnt, 31);
                        {
                            int pn = (int)(ex & 0xffff), pb = (int)((ex >> 16) & 0xffff), ps = (int)(ex >> 32);
                            unsigned short tag = (unsigned short)(lane << 5);
                            unsigned m = mn;
                            while (m) {
                                int jj = __ffs(m) - 1;
                                m &= m - 1;
                                S.q[0][pn++] = tag | jj;
                            }
                            m = mb;
                            while (m) {
                                int jj = __ffs(m) - 1;
                                m &= m - 1;
                                S.q[1][pb++] = tag | jj;
                            }
                            m = ms;
                            while (m) {
                                int jj = __ffs(m) - 1;
                                m &= m - 1;
                                S.q[2][ps++] = tag | jj;
                            }
                        }
                        __syncwarp();
                        const int nn = (int)(tot & 0xffff), nbq = (int)((tot >> 16) & 0xffff), nsq = (int)(tot >> 32);
                        // screened pairs: T(r) polynomial of S - R_d only.  Lane l takes the
                        // contiguous block [l K, (l+1) K) of the target-major queue and sums
                        // runs of one target in registers: a target that starts inside the
                        // block is added by this lane alone; the block's first target (which
                        // may continue from earlier lanes) goes through one segmented reduction.
                        {
                            const int K = (nn + 31) >> 5;
                            const int eb = min(lane * K, nn), ee = min(eb + K, nn);
                            int cur = -1, first = -1;
                            float a0 = 0, a1 = 0, a2 = 0, f0 = 0, f1 = 0, f2 = 0;
                            for (int ei = eb; ei < ee; ei++) {
                                const int qv = S.q[0][ei], t = qv >> 5, jj = qv & 31;
                                float4 p = S.s_hi[jj], pl = S.s_lo[jj], f = S.s_f[jj];
                                float4 a = S.t_hi[t], al = S.t_lo[t];
                                float dx = (a.x - p.x) + (al.x - pl.x);
                                float dy = (a.y - p.y) + (al.y - pl.y);
                                float dz = (a.z - p.z) + (al.z - pl.z);
                                float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                float ri = rsqrtf(r2);
                                ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);
                                float r = r2 * ri;
                                const float2 T12 = horner2<NP>(c12, fmaf(r, tds, tdo));
                                float H1 = T12.x * ri, H2 = T12.y * (ri * ri * ri);
                                float g = H2 * fmaf(f.x, dx, fmaf(f.y, dy, f.z * dz));
                                const float v0 = fmaf(H1, f.x, g * dx);
                                const float v1 = fmaf(H1, f.y, g * dy);
                                const float v2 = fmaf(H1, f.z, g * dz);
                                if (t != cur) {
                                    if (cur >= 0) {
                                        if (first < 0) {
                                            first = cur;
                                            f0 = a0;
                                            f1 = a1;
                                            f2 = a2;
                                        } else {
                                            S.acc[0][cur] += a0;
                                            S.acc[1][cur] += a1;
                                            S.acc[2][cur] += a2;
                                        }
                                    }
                                    cur = t;
                                    a0 = v0;
                                    a1 = v1;
                                    a2 = v2;
                                } else {
                                    a0 += v0;
                                    a1 += v1;
                                    a2 += v2;
                                }
                            }
                            if (cur >= 0) {
                                if (first < 0) {
                                    first = cur;
                                    f0 = a0;
                                    f1 = a1;
                                    f2 = a2;
                                } else {
                                    S.acc[0][cur] += a0;
                                    S.acc[1][cur] += a1;
                                    S.acc[2][cur] += a2;
                                }
                            }
                            __syncwarp();
                            if (nn > 0) segment_reduce_add(f0, f1, f2, first >= 0 ? first : -1 - lane, lane, S.acc);
                        }
                        // near pairs (r < r_mid): the blob piece (R_eps - R_d itself) inside the
                        // blob region, else the near piece of S - R_d
                        for (int e0 = 0; e0 < nbq; e0 += 32) {
                            const int ei = e0 + lane;
                            float v0 = 0, v1 = 0, v2 = 0;
                            int key = -1 - lane;
                            if (ei < nbq) {
                                const int qv = S.q[1][ei], t = qv >> 5, jj = qv & 31;
                                key = t;
                                float4 p = S.s_hi[jj], pl = S.s_lo[jj], f = S.s_f[jj];
                                float4 a = S.t_hi[t], al = S.t_lo[t];
                                float dx = (a.x - p.x) + (al.x - pl.x);
                                float dy = (a.y - p.y) + (al.y - pl.y);
                                float dz = (a.z - p.z) + (al.z - pl.z);
                                float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                float ri = rsqrtf(r2);
                                ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);
                                float r = r2 * ri;
                                float H1, H2;
                                if (r2 < rs2) {
                                    const float2 h = cheb2(S.tb, nbp, fmaf(r, tbs, tbo));
                                    H1 = h.x;
                                    H2 = h.y * (ri * ri);
                                } else {
                                    const float2 T12 = cheb2(S.tn, nnp, fmaf(r, tns, tno));
                                    H1 = T12.x * ri;
                                    H2 = T12.y * (ri * ri * ri);
                                }
                                float g = H2 * fmaf(f.x, dx, fmaf(f.y, dy, f.z * dz));
                                v0 = fmaf(H1, f.x, g * dx);
                                v1 = fmaf(H1, f.y, g * dy);
                                v2 = fmaf(H1, f.z, g * dz);
                            }
                            segment_reduce_add(v0, v1, v2, key, lane, S.acc);
                        }
                        // series pairs (r < r_tiny): FP64 series of R_eps - R_d, FP64 sums
                        for (int e0 = 0; e0 < nsq; e0 += 32) {
                            const int ei = e0 + lane;
                            if (ei < nsq) {
                                const int qv = S.q[2][ei], t = qv >> 5, jj = qv & 31;
                                float4 p = S.s_hi[jj], pl = S.s_lo[jj], f = S.s_f[jj];
                                float4 a = S.t_hi[t], al = S.t_lo[t];
                                double dx = (double)(a.x - p.x) + (double)(al.x - pl.x);
                                double dy = (double)(a.y - p.y) + (double)(al.y - pl.y);
                                double dz = (double)(a.z - p.z) + (double)(al.z - pl.z);
                                double rr = dx * dx + dy * dy + dz * dz;
                                double H1, H2;
                                if (T.blob) {
                                    series_H(T, rr, H1, H2);
                                } else if (rr == 0.0) {
                                    H1 = T.self1;  // coincident points, eps = 0: the reference's r -> 0 limit
                                    H2 = 0;
                                } else {  // eps = 0, nearly coincident: singular kernel from the near piece
                                    float r2f = (float)rr, ri = rsqrtf(r2f);
                                    ri = ri * fmaf(-0.5f * r2f * ri, ri, 1.5f);
                                    const float2 T12 = cheb2(S.tn, nnp, fmaf(r2f * ri, tns, tno));
                                    H1 = (double)(T12.x * ri);
                                    H2 = (double)(T12.y * (ri * ri * ri));
                                }
                                double fd = f.x * dx + f.y * dy + f.z * dz;
                                atomicAdd(&S.acc64[0][t], H1 * f.x + H2 * fd * dx);
                                atomicAdd(&S.acc64[1][t], H1 * f.y + H2 * fd * dy);
                                atomicAdd(&S.acc64[2][t], H1 * f.z + H2 * fd * dz);
                            }
                        }
                        __syncwarp();
                        kahan_add(s0, k0, S.acc[0][lane]);
                        kahan_add(s1, k1, S.acc[1][lane]);
                        kahan_add(s2, k2, S.acc[2][lane]);
                        S.acc[0][lane] = 0.f;
                        S.acc[1][lane] = 0.f;
                        S.acc[2][lane] = 0.f;
                        __syncwarp();
                    }
                }
            }
        }
        if (active) {  // the item's part of the target's sum (other column groups add theirs)
            size_t o = 3 * (size_t)tidx;
            atomicAdd(u_real + o, ((double)s0 - (double)k0) + S.acc64[0][lane]);
            atomicAdd(u_real + o + 1, ((double)s1 - (double)k1) + S.acc64[1][lane]);
            atomicAdd(u_real + o + 2, ((double)s2 - (double)k2) + S.acc64[2][lane]);
        }
        S.acc64[0][lane] = 0.0;
        S.acc64[1][lane] = 0.0;
        S.acc64[2][lane] = 0.0;
        __syncwarp();
    }
}

void launch_real_mixed(int npoly, const PbInst* inst, const PbTables* tab, const int4* items, const int* nitems_ptr,
                       int nitems_max,
                       const float4* spos_hi, const float4* spos_lo, const float4* sfrc, const int* src_start,
                       const float4* tpos_hi, const float4* tpos_lo, int ntgt_cap, double* u_real, int* counter,
                       int nsm, cudaStream_t s)
{
    if (nitems_max <= 0) return;
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    cudaMemsetAsync(u_real, 0, 3 * sizeof(double) * (size_t)ntgt_cap, s);
    int blocks = nsm * 8;
    int need = (nitems_max + kRealWarps - 1) / kRealWarps;
    if (blocks > need) blocks = need;
#define PB_LAUNCH_REAL(NP)                                                                                            \
    k_real_mixed<NP><<<blocks, kRealWarps * 32, 0, s>>>(inst, tab, items, nitems_ptr, spos_hi, spos_lo, sfrc,        \
                                                         src_start,                                                  \
                                                         tpos_hi, tpos_lo, u_real, counter, nitems_max)
    if (npoly <= 16)
        PB_LAUNCH_REAL(16);
    else if (npoly <= 20)
        PB_LAUNCH_REAL(20);
    else if (npoly <= 24)
        PB_LAUNCH_REAL(24);
    else if (npoly <= 26)
        PB_LAUNCH_REAL(26);
    else
        PB_LAUNCH_REAL(28);
#undef PB_LAUNCH_REAL
}

__global__ void __launch_bounds__(kRealWarps * 32)
    k_real_fp64(const PbInst* __restrict__ inst, const PbTables* __restrict__ tab, const int4* __restrict__ items,
                const int* __restrict__ nitems_ptr, const Dbl4* __restrict__ spos, const Dbl4* __restrict__ sfrc,
                const int* __restrict__ src_start, const Dbl4* __restrict__ tpos, double* __restrict__ u,
                int* __restrict__ counter, int item_cap)
{
    __shared__ Dbl4 sh_p[kRealWarps][32];
    __shared__ Dbl4 sh_f[kRealWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nitems = min(*nitems_ptr, item_cap);
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
        const bool active = lane < F.count;
        const int tidx = F.first + (active ? lane : 0);
        const int self_src = I.same ? tidx - I.tgt_off + I.src_off : -1;
        Dbl4 tp = tpos[tidx];
        if (!active) tp.x = tp.y = tp.z = 3.0e300;  // inactive lanes pair with nothing
        double v0 = 0, v1 = 0, v2 = 0;
        const int ny1 = 2 * I.S[1] + 1, ncol = (2 * I.S[0] + 1) * ny1;
        const int csplit = max(1, I.csplit);
        for (int col = F.group; col < ncol; col += csplit) {
            const int o0 = col / ny1 - I.S[0], o1 = col % ny1 - I.S[1];
            int g0 = F.c0 + o0;
            int w0 = ((g0 % I.nc[0]) + I.nc[0]) % I.nc[0];
            double sh0 = (double)((g0 - w0) / I.nc[0]) * I.L[0];
            {
                int g1 = F.c1 + o1;
                int w1 = ((g1 % I.nc[1]) + I.nc[1]) % I.nc[1];
                double sh1 = (double)((g1 - w1) / I.nc[1]) * I.L[1];
                int row = I.cell_off + (w0 * I.nc[1] + w1) * I.nc[2];
                int g2 = F.za - I.S[2];
                const int g2end = F.zb + I.S[2];
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
        if (active) {  // the item's part of the target's sum (other column groups add theirs)
            size_t o = 3 * (size_t)tidx;
            atomicAdd(u + o, v0);
            atomicAdd(u + o + 1, v1);
            atomicAdd(u + o + 2, v2);
        }
    }
}

void launch_real_fp64(const PbInst* inst, const PbTables* tab, const int4* items, const int* nitems_ptr,
                      int nitems_max, const Dbl4* spos, const Dbl4* sfrc, const int* src_start,
                      const Dbl4* tpos, int ntgt_cap, double* u, int* counter, int nsm, cudaStream_t s)
{
    if (nitems_max <= 0) return;
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    cudaMemsetAsync(u, 0, 3 * sizeof(double) * (size_t)ntgt_cap, s);
    int blocks = nsm * 8;
    int need = (nitems_max + kRealWarps - 1) / kRealWarps;
    if (blocks > need) blocks = need;
    k_real_fp64<<<blocks, kRealWarps * 32, 0, s>>>(inst, tab, items, nitems_ptr, spos, sfrc, src_start, tpos, u,
                                                   counter, nitems_max);
}

}  // namespace pb
