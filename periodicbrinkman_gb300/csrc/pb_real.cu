// Real-space Ewald sum over a device-built cell list.
//
// Work item = (instance, cell row (c0, c1), z-range [za, zb] of at most
// kItemCells cells, up to 32 consecutive sorted targets, a group of the stencil's
// columns), one warp per item, items pulled from a global counter by a
// persistent grid.  Each lane owns one target.  Each stencil column is cut to
// the part of the cutoff ball around the targets' box; its contiguous z-runs
// of the cell-sorted source array are gathered as segments and streamed
// through shared memory 32 sources at a time, dropping sources beyond rc of
// the box.  Mixed precision: each lane classifies its 32 candidate pairs
// (inside the cutoff / below r_mid), the warp compacts the pairs inside the
// cutoff into a target-major queue, and every lane then evaluates a block of
// it, so the FMA pipe sees full warps; per-target sums of each chunk are
// formed by one segmented warp reduction (no atomics).  Pairs below r_mid
// (blob, near and series pieces) are queued per warp and evaluated 32 at a
// time.
//
// Mixed precision (k_real_mixed): positions are FP32 hi/lo pairs re-expressed
// in the frame of the target cell (error-free TwoSum), so displacements carry
// FP32 relative accuracy even at r << cell size; the pair kernel is the FP32
// polynomial T(r) of the instance tables (FMA only); per-chunk partial sums are
// Kahan-accumulated; pairs below r_tiny use the FP64 series, added straight to
// the target's FP64 sum.  The self pair of targets that are the sources is skipped here
// and added in FP64 by the combine kernel (R_eps(0) - R_d(0)) f_i.
//
// FP64 (k_real_fp64): beyond r_mid an FP64 Chebyshev series of the screened
// kernel (fitted on the host to the reference's closed forms), below it the
// closed forms themselves (cuda/periodicBrinkman.h:85-176) in double precision,
// FP64 series below r_tiny.  The in-cutoff pairs of each chunk are compacted
// and evaluated 32 at a time, so the FP64 pipe sees full warps.
#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

constexpr int kRealWarps = 4;

constexpr int kMaxReach = 15;  // stencil reach S per axis
constexpr int kZTab = kItemCells + 2 * kMaxReach;

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
    short wx[2 * kMaxReach + 1], wy[2 * kMaxReach + 1], wz[kZTab];  // wrapped cells (< 128)
    unsigned zx, zy, zz[2];  // bit k: the image shift of offset k is zero
};
static_assert(2 * kMaxReach + 1 <= 32 && kZTab <= 64, "zero-shift bitmasks");

// c h - s L as an FP32 hi/lo pair (double-float arithmetic: the products are
// split exactly by FMAs), for a cell index c and an image shift count s.
__device__ __forceinline__ void frame_offset(const PbInst& I, int ax, int c, int sc, float& hi, float& lo)
{
    const float cf = (float)c, sf = (float)sc;
    const float p1 = cf * I.hch[ax], e1 = fmaf(cf, I.hch[ax], -p1);
    const float p2 = sf * I.Lh[ax], e2 = fmaf(sf, I.Lh[ax], -p2);
    float s, er;
    two_sum(p1, -p2, s, er);
    const float l = er + ((e1 + cf * I.hcl[ax]) - (e2 + sf * I.Ll[ax]));
    hi = s + l;
    lo = l - (hi - s);
}

__device__ __forceinline__ void fill_frame_tabs(const PbInst& I, const ItemFrame& F, FrameTabs& T, int lane)
{
    const int nx = 2 * I.S[0] + 1, ny = 2 * I.S[1] + 1, nz = F.zb - F.za + 2 * I.S[2] + 1;
    if (lane == 0) {
        T.zx = 0u;
        T.zy = 0u;
        T.zz[0] = 0u;
        T.zz[1] = 0u;
    }
    __syncwarp();
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
        int w, sc;  // wrapped cell and image shift count (one wrap at most, unless the box has few cells)
        if (g >= 0 && g < n) {
            w = g;
            sc = 0;
        } else if (g < 0 && g >= -n) {
            w = g + n;
            sc = -1;
        } else if (g >= n && g < 2 * n) {
            w = g - n;
            sc = 1;
        } else {
            w = ((g % n) + n) % n;
            sc = (g - w) / n;
        }
        float hi, lo;  // Q = O - sc L, O = the frame cell's corner
        frame_offset(I, ax, ax == 0 ? F.c0 : ax == 1 ? F.c1 : F.za, sc, hi, lo);
        if (ax == 0) {
            T.qx[k] = make_float2(hi, lo);
            T.wx[k] = (short)w;
            if (sc == 0) atomicOr(&T.zx, 1u << k);
        } else if (ax == 1) {
            T.qy[k] = make_float2(hi, lo);
            T.wy[k] = (short)w;
            if (sc == 0) atomicOr(&T.zy, 1u << k);
        } else {
            T.qz[k] = make_float2(hi, lo);
            T.wz[k] = (short)w;
            if (sc == 0) atomicOr(&T.zz[k >> 5], 1u << (k & 31));
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
constexpr int kSeg = 64;   // candidate segments gathered before they are streamed
constexpr int kNear = 40;  // deferred near pairs (evaluated 32 at a time; <= 31 wait)

struct __align__(16) RealWarpSmem {
    float4 s_hi[32], s_lo[32], s_f[32];     // staged sources: frame-relative hi, lo; force
    float4 t_hi[32], t_lo[32];              // the item's targets: frame-relative hi, lo
    float4 nq_h[kNear], nq_l[kNear], nq_f[kNear];  // deferred near pairs: displacement hi (target in w), lo; force
    float c_x[32], c_y[32], c_z[32];        // staged sources, hi parts by axis (classification)
    float acc[3][32];                       // per-target partial sums of the current chunk
    float ks[6][32];                        // per-target Kahan sums (3) and compensations (3) of the item
    unsigned selfm[32];                     // per target: the staged candidate that is its own source
    int sg_b[kSeg], sg_n[kSeg], sg_pre[kSeg], sg_meta[kSeg];  // segments: first source, count, prefix, frame
    float box[6];                           // the item's targets: frame-relative bounding box (hi parts)
    int nq_n;                               // deferred near pairs waiting
    unsigned short q[1024];                 // in-cutoff pairs of a chunk, target-major (t << 5 | j)
    float2 tn[kMaxCheb];                    // near piece (T1, T2) of the current instance
    float2 tb[kMaxCheb];                    // blob piece (H1, r^2 H2) of the current instance
    FrameTabs ft;                           // the current item's frame tables
    struct {
        float rtiny2, rs2, tbs, tbo, tns, tno;
        int nbp, nnp;
    } rk;                                   // constants of the rare pieces of the current instance
};

// Warp-wide exclusive prefix sum.
__device__ __forceinline__ int warp_excl_scan(int v, int lane)
{
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    return x - v;
}

// Order-preserving map of floats to ints (for warp min/max reductions).
__device__ __forceinline__ int float_key(float f)
{
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float key_float(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

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

// The instance's constants of the common path, held by each lane.
struct MixedConsts {
    float tds, tdo, rc2, rare2;
};

// A pair below r_mid: the blob piece (R_eps - R_d itself) inside the blob
// region, else the near piece of S - R_d; below r_tiny (or at r = 0) the FP64
// series, added to the target's FP64 sum u_t[3 t..] in global memory (then
// v = 0).
__device__ __forceinline__ void rare_pair(RealWarpSmem& S, const PbTables& T, float4 h, float4 l, float4 f, int t,
                                          float& v0, float& v1, float& v2, double* __restrict__ u_t)
{
    const auto& K = S.rk;
    const float dx = h.x + l.x, dy = h.y + l.y, dz = h.z + l.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    v0 = v1 = v2 = 0.f;
    if ((r2 < K.rtiny2) | (r2 == 0.f)) {
        const double ddx = (double)h.x + (double)l.x, ddy = (double)h.y + (double)l.y, ddz = (double)h.z + (double)l.z;
        const double rr = ddx * ddx + ddy * ddy + ddz * ddz;
        double H1, H2;
        if (T.blob) {
            series_H(T, rr, H1, H2);
        } else if (rr == 0.0) {
            H1 = T.self1;  // coincident points, eps = 0: the reference's r -> 0 limit
            H2 = 0;
        } else {  // eps = 0, nearly coincident: singular kernel from the near piece
            float r2f = (float)rr, ri = rsqrtf(r2f);
            ri = ri * fmaf(-0.5f * r2f * ri, ri, 1.5f);
            const float2 T12 = cheb2(S.tn, K.nnp, fmaf(r2f * ri, K.tns, K.tno));
            H1 = (double)(T12.x * ri);
            H2 = (double)(T12.y * (ri * ri * ri));
        }
        const double fd = f.x * ddx + f.y * ddy + f.z * ddz;
        atomicAdd(u_t + 3 * t, H1 * f.x + H2 * fd * ddx);
        atomicAdd(u_t + 3 * t + 1, H1 * f.y + H2 * fd * ddy);
        atomicAdd(u_t + 3 * t + 2, H1 * f.z + H2 * fd * ddz);
        return;
    }
    float ri = rsqrtf(r2);
    ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);
    const float r = r2 * ri;
    float H1, H2;
    if (r2 < K.rs2) {
        const float2 b = cheb2(S.tb, K.nbp, fmaf(r, K.tbs, K.tbo));
        H1 = b.x;
        H2 = b.y * (ri * ri);
    } else {
        const float2 T12 = cheb2(S.tn, K.nnp, fmaf(r, K.tns, K.tno));
        H1 = T12.x * ri;
        H2 = T12.y * (ri * ri * ri);
    }
    const float g = H2 * fmaf(f.x, dx, fmaf(f.y, dy, f.z * dz));
    v0 = fmaf(H1, f.x, g * dx);
    v1 = fmaf(H1, f.y, g * dy);
    v2 = fmaf(H1, f.z, g * dz);
}

// Evaluate the `n` (<= 32) deferred near pairs [end - n, end), one per lane,
// into the per-target accumulators: each lane writes its pair's contribution
// over the entry, then lane t sums the entries of target t (no atomics; shared
// float atomics measured slower here).
__device__ __forceinline__ void near_flush(RealWarpSmem& S, const PbTables& T, int end, int n, int lane,
                                           double* __restrict__ u_t)
{
    const int e0 = end - n;
    if (lane < n) {
        const int e = e0 + lane;
        const float4 h = S.nq_h[e];
        const int t = __float_as_int(h.w);
        float v0, v1, v2;
        rare_pair(S, T, h, S.nq_l[e], S.nq_f[e], t, v0, v1, v2, u_t);
        S.nq_h[e] = make_float4(v0, v1, v2, h.w);
    }
    __syncwarp();
    float a0 = 0.f, a1 = 0.f, a2 = 0.f;
    for (int i = 0; i < n; i++) {
        const float4 w = S.nq_h[e0 + i];
        if (__float_as_int(w.w) == lane) {
            a0 += w.x;
            a1 += w.y;
            a2 += w.z;
        }
    }
    S.acc[0][lane] += a0;
    S.acc[1][lane] += a1;
    S.acc[2][lane] += a2;
    __syncwarp();
}

// Kahan-add the chunk's per-target sums into the item's sums; clear them.
__device__ __forceinline__ void chunk_sums(RealWarpSmem& S, int lane)
{
#pragma unroll
    for (int c = 0; c < 3; c++) {
        float sc = S.ks[c][lane], kc = S.ks[3 + c][lane];
        kahan_add(sc, kc, S.acc[c][lane]);
        S.ks[c][lane] = sc;
        S.ks[3 + c][lane] = kc;
        S.acc[c][lane] = 0.f;
    }
}

// Segment of candidate pos + lane, without a search: the segment holding
// `pos` plus the segment starts in (pos, pos + lane] (at most 64 segments,
// two per lane).  `pos` is the same for the whole warp.
__device__ __forceinline__ int candidate_segment(const RealWarpSmem& S, int nseg, int pos, int lane)
{
    const int ka = lane, kb = lane + 32;
    const int pa = ka < nseg ? S.sg_pre[ka] : 0x7fffffff, pb = kb < nseg ? S.sg_pre[kb] : 0x7fffffff;
    const int k0 = __popc(__ballot_sync(kFull, pa <= pos)) + __popc(__ballot_sync(kFull, pb <= pos)) - 1;
    const unsigned bits = (pa > pos && pa - pos < 32 ? 1u << (pa - pos) : 0u) |
                          (pb > pos && pb - pos < 32 ? 1u << (pb - pos) : 0u);
    const unsigned starts = __reduce_or_sync(kFull, bits);
    return k0 + __popc(starts & ((2u << lane) - 2u));
}

// Stream the gathered candidate segments through the warp 32 sources at a
// time: stage, classify against the item's targets, queue the pairs inside
// the cutoff target-major and evaluate them (far polynomial; pairs below
// r_mid are deferred to the near queue).
template <int NP>
__device__ __forceinline__ void stream_segments(RealWarpSmem& S, const PbInst& I, const PbTables& T,
                                                const MixedConsts& K, const float2 (&c12)[NP], const ItemFrame& F,
                                                int nseg, int lane, const float4* __restrict__ spos_hi,
                                                const float4* __restrict__ spos_lo, const float4* __restrict__ sfrc,
                                                double* __restrict__ u_real)
{
    // exclusive prefix of the segment counts (two segments per lane)
    int total;
    {
        const int a = 2 * lane, b = 2 * lane + 1;
        const int n0 = a < nseg ? S.sg_n[a] : 0, n1 = b < nseg ? S.sg_n[b] : 0;
        const int ex = warp_excl_scan(n0 + n1, lane);
        if (a < nseg) S.sg_pre[a] = ex;
        if (b < nseg) S.sg_pre[b] = ex + n0;
        total = __shfl_sync(kFull, ex + n0 + n1, 31);
    }
    __syncwarp();
    const int self_shift = I.same ? I.tgt_off - I.src_off - F.first : 0;
    const unsigned lt = (1u << lane) - 1u;
    const float keep2 = K.rc2 * 1.0001f;
    // Chunks of 32 sources that lie within rc of the targets' box: candidates
    // are fetched 32 at a time and the others (about 30% of a column's cells)
    // are dropped before any pair is tested.
    int pos = 0;
    while (pos < total) {
        int fill = 0;
        while (fill < 32 && pos < total) {
            const int p = pos + lane;
            const int seg = candidate_segment(S, nseg, pos, lane);
            bool keep = false, zs = false;
            int j = 0;
            float p3[3] = {0.f, 0.f, 0.f}, l3[3] = {0.f, 0.f, 0.f};
            float4 fj = make_float4(0.f, 0.f, 0.f, 0.f);
            if (p < total) {
                j = S.sg_b[seg] + (p - S.sg_pre[seg]);
                const int meta = S.sg_meta[seg];
                const int i0 = meta & 31, i1 = (meta >> 5) & 31, i2 = meta >> 10;
                const float2 qx = S.ft.qx[i0], qy = S.ft.qy[i1], qz = S.ft.qz[i2];
                const float qh[3] = {qx.x, qy.x, qz.x}, ql[3] = {qx.y, qy.y, qz.y};
                const float4 ph = spos_hi[j], pl = spos_lo[j];
                fj = sfrc[j];  // loaded with the position (not after the test): one round of latency
                const float xh[3] = {ph.x, ph.y, ph.z}, xl[3] = {pl.x, pl.y, pl.z};
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    float sv, er;
                    two_sum(xh[a], -qh[a], sv, er);
                    p3[a] = sv;
                    l3[a] = er + (xl[a] - ql[a]);
                }
                float d2 = 0.f;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const float da = fmaxf(0.f, fmaxf(S.box[a] - p3[a], p3[a] - S.box[3 + a]));
                    d2 = fmaf(da, da, d2);
                }
                keep = d2 < keep2;
                zs = I.same && ((S.ft.zx >> i0) & (S.ft.zy >> i1) & (S.ft.zz[i2 >> 5] >> (i2 & 31)) & 1u);
            }
            const unsigned bal = __ballot_sync(kFull, keep);
            const int need = 32 - fill, k = __popc(bal), rank = __popc(bal & lt);
            int adv = min(32, total - pos);
            if (k > need) adv = __ffs(__ballot_sync(kFull, keep && rank == need - 1));  // through the last one taken
            if (keep && rank < need) {
                const int slot = fill + rank;
                S.s_hi[slot] = make_float4(p3[0], p3[1], p3[2], 0.f);
                S.s_lo[slot] = make_float4(l3[0], l3[1], l3[2], 0.f);
                S.s_f[slot] = fj;
                S.c_x[slot] = p3[0];
                S.c_y[slot] = p3[1];
                S.c_z[slot] = p3[2];
                if (zs) {  // a target's own source (added by the combine kernel)
                    const int ts = j + self_shift;
                    if (ts >= 0 && ts < F.count) S.selfm[ts] = 1u << slot;
                }
            }
            fill += min(k, need);
            pos += adv;
        }
        if (lane >= fill) {  // padding: far from every target, active (finite) or not (+3e30)
            S.c_x[lane] = -3.0e30f;
            S.c_y[lane] = -3.0e30f;
            S.c_z[lane] = -3.0e30f;
        }
        __syncwarp();
        // candidate pairs of this lane's target inside the cutoff and below r_mid (two per
        // packed FP32x2 operation)
        unsigned mi = 0, mr = 0;
        {
            const float4 tt = S.t_hi[lane];
            const float2 ntx = make_float2(-tt.x, -tt.x), nty = make_float2(-tt.y, -tt.y),
                         ntz = make_float2(-tt.z, -tt.z);
#pragma unroll
            for (int jj = 0; jj < 32; jj += 2) {
                const float2 dx = __fadd2_rn(*reinterpret_cast<const float2*>(&S.c_x[jj]), ntx);
                const float2 dy = __fadd2_rn(*reinterpret_cast<const float2*>(&S.c_y[jj]), nty);
                const float2 dz = __fadd2_rn(*reinterpret_cast<const float2*>(&S.c_z[jj]), ntz);
                float2 r2 = __fmul2_rn(dx, dx);
                r2 = __ffma2_rn(dy, dy, r2);
                r2 = __ffma2_rn(dz, dz, r2);
                if (r2.x < K.rc2) mi |= 1u << jj;
                if (r2.y < K.rc2) mi |= 2u << jj;
                if (r2.x < K.rare2) mr |= 1u << jj;
                if (r2.y < K.rare2) mr |= 2u << jj;
            }
        }
        mi &= ~S.selfm[lane];
        mr &= ~S.selfm[lane];
        S.selfm[lane] = 0u;
        mi &= ~mr;
        // target-major queues: pairs inside the cutoff from the front of q, pairs
        // below r_mid from its back (the two are disjoint pairs of the chunk)
        const int cnt = __popc(mi) | (__popc(mr) << 16);
        int ex = warp_excl_scan(cnt, lane);
        const int tot = __shfl_sync(kFull, ex + cnt, 31);
        const int nn = tot & 0xffff, nr = tot >> 16;
        {
            const unsigned short tag = (unsigned short)(lane << 5);
            int pn = ex & 0xffff, pr = 1023 - (ex >> 16);
            {  // lowest and highest set bits per step: half the dependent iterations of one bit per step
                int pe = pn + __popc(mi) - 1;
                for (unsigned m = mi; m;) {
                    const int lo = __ffs(m) - 1, hi = 31 - __clz(m);
                    S.q[pn++] = tag | lo;
                    if (hi != lo) S.q[pe--] = tag | hi;
                    m &= ~((1u << lo) | (1u << hi));
                }
            }
            for (unsigned m = mr; m; m &= m - 1) S.q[pr--] = tag | (__ffs(m) - 1);
        }
        __syncwarp();
        // pairs below r_mid join the near queue (<= 31 waiting), which is
        // evaluated whenever it holds 32
        for (int r0 = 0; r0 < nr;) {
            const int nq = S.nq_n;
            const int k = min(nr - r0, kNear - nq);
            __syncwarp();
            for (int i = lane; i < k; i += 32) {
                const int qv = S.q[1023 - (r0 + i)], t = qv >> 5, jj = qv & 31;
                const float4 p = S.s_hi[jj], pl = S.s_lo[jj], a = S.t_hi[t], al = S.t_lo[t];
                S.nq_h[nq + i] = make_float4(a.x - p.x, a.y - p.y, a.z - p.z, __int_as_float(t));
                S.nq_l[nq + i] = make_float4(al.x - pl.x, al.y - pl.y, al.z - pl.z, 0.f);
                S.nq_f[nq + i] = S.s_f[jj];
            }
            __syncwarp();
            int n = nq + k;
            while (n >= 32) {
                near_flush(S, T, n, 32, lane, u_real + 3 * (size_t)F.first);
                n -= 32;
            }
            if (lane == 0) S.nq_n = n;
            __syncwarp();
            r0 += k;
        }
        // Lane l takes the contiguous block [l K, (l+1) K) of the queue and sums runs
        // of one target in registers: a target that starts inside the block is added
        // by this lane alone; the block's first target (which may continue from
        // earlier lanes) goes through one segmented reduction.
        {
            const int KB = (nn + 31) >> 5;
            const int eb = min(lane * KB, nn), ee = min(eb + KB, nn);
            int cur = -1, first = -1;
            float a0 = 0, a1 = 0, a2 = 0, f0 = 0, f1 = 0, f2 = 0;
            int qn = eb < ee ? S.q[eb] : 0;  // the next entry, loaded one pair ahead
            for (int ei = eb; ei < ee; ei++) {
                const int qv = qn, t = qv >> 5, jj = qv & 31;
                if (ei + 1 < ee) qn = S.q[ei + 1];
                const float4 p = S.s_hi[jj], pl = S.s_lo[jj], f = S.s_f[jj];
                const float4 a = S.t_hi[t], al = S.t_lo[t];
                const float dx = (a.x - p.x) + (al.x - pl.x);
                const float dy = (a.y - p.y) + (al.y - pl.y);
                const float dz = (a.z - p.z) + (al.z - pl.z);
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                float ri = rsqrtf(r2);
                ri = ri * fmaf(-0.5f * r2 * ri, ri, 1.5f);
                const float r = r2 * ri;
                const float2 T12 = horner2<NP>(c12, fmaf(r, K.tds, K.tdo));
                const float H1 = T12.x * ri, H2 = T12.y * (ri * ri * ri);
                const float g = H2 * fmaf(f.x, dx, fmaf(f.y, dy, f.z * dz));
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
        __syncwarp();

        chunk_sums(S, lane);
        __syncwarp();
    }
}

// Four blocks of four warps per SM (128 registers; 44.7 KB of shared memory a
// block, which leaves about 45 KB of L1).  Five blocks (96 registers, with
// spills) measured 8% slower.
template <int NP>
__global__ void __launch_bounds__(kRealWarps * 32, 4)
    k_real_mixed(const PbInst* __restrict__ inst, const PbTables* __restrict__ tab, const int4* __restrict__ items,
                 const int* __restrict__ nitems_ptr, const float4* __restrict__ spos_hi, const float4* __restrict__ spos_lo,
                 const float4* __restrict__ sfrc, const int* __restrict__ src_start, const float4* __restrict__ tpos_hi, const float4* __restrict__ tpos_lo, double* __restrict__ u_real,
                 int* __restrict__ counter, int item_cap)
{
    __shared__ RealWarpSmem smem_all[kRealWarps];
    RealWarpSmem& S = smem_all[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;

    const int nitems = min(*nitems_ptr, item_cap);
    float2 c12[NP];
    int cur_q = -1;
    MixedConsts K{};
#pragma unroll
    for (int c = 0; c < 3; c++) {
        S.acc[c][lane] = 0.f;
    }
    S.selfm[lane] = 0u;
    if (lane == 0) S.nq_n = 0;
    __syncwarp();

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
            K.tds = T.td_scale;
            K.tdo = T.td_off;
            K.rc2 = T.rc2;
            K.rare2 = T.rm2;  // below r_mid: the near and blob pieces (and r = 0)
            if (lane == 0) {
                S.rk.rs2 = T.rs2;
                S.rk.tns = T.tn_scale;
                S.rk.tno = T.tn_off;
                S.rk.nnp = T.nn > 0 ? T.nn : 1;
                S.rk.rtiny2 = T.rtiny2f;
                S.rk.tbs = T.tb_scale;
                S.rk.tbo = T.tb_off;
                S.rk.nbp = T.nb > 0 ? T.nb : 1;
            }
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
        float th[3];
        {
            float4 ph = tpos_hi[tidx], pl = tpos_lo[tidx];
            float xh[3] = {ph.x, ph.y, ph.z}, xl[3] = {pl.x, pl.y, pl.z}, tl[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                float oh, ol, s, e;
                frame_offset(I, a, a == 0 ? F.c0 : a == 1 ? F.c1 : F.za, 0, oh, ol);
                two_sum(xh[a], -oh, s, e);
                th[a] = active ? s : 3.0e30f;  // inactive lanes pair with nothing
                tl[a] = e + (xl[a] - ol);
            }
            S.t_hi[lane] = make_float4(th[0], th[1], th[2], 0.f);
            S.t_lo[lane] = make_float4(tl[0], tl[1], tl[2], 0.f);
            // bounding box of the item's targets (hi parts; the margin below covers the rest)
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const int kmin = __reduce_min_sync(kFull, float_key(active ? th[a] : 3.0e30f));
                const int kmax = __reduce_max_sync(kFull, float_key(active ? th[a] : -3.0e30f));
                if (lane == 0) {
                    S.box[a] = key_float(kmin);
                    S.box[3 + a] = key_float(kmax);
                }
            }
        }
#pragma unroll
        for (int c = 0; c < 6; c++) S.ks[c][lane] = 0.f;
        __syncwarp();

        // The item's stencil columns, 32 at a time (a lane per column): the
        // column's part of the cutoff ball around the targets' box is a z-range,
        // taken at cell granularity (cells are rc/4 along z); its cells are cut
        // into runs at the periodic wrap.  The runs are gathered as segments and
        // streamed through the warp in full chunks of 32 sources.
        const int ny1 = 2 * I.S[1] + 1, ncol = (2 * I.S[0] + 1) * ny1;
        const int csplit = max(1, I.csplit);
        const int ncg = (ncol - F.group + csplit - 1) / csplit;
        const float h0 = (float)I.h[0], h1 = (float)I.h[1], ih2 = 1.f / (float)I.h[2];
        const float marg = 4e-6f * fmaxf((float)I.L[0], fmaxf((float)I.L[1], (float)I.L[2]));
        const int nzt = F.zb - F.za + 2 * I.S[2] + 1;
        // gather segments until the list could overflow in the next round, stream
        // them (one call site keeps the hot loop once in the instruction cache),
        // repeat; per-lane column cursors persist across the streaming
        int nseg = 0, kb = 0;
        bool open = false;
        int i0 = 0, i1 = 0, i2 = 1, i2b = 0, row = 0;
        while (true) {
            while (true) {
                if (!open) {
                    if (kb >= ncg) break;
                    i2 = 1;
                    i2b = 0;
                    if (kb + lane < ncg) {
                        const int col = F.group + (kb + lane) * csplit;
                        i0 = col / ny1;
                        i1 = col - i0 * ny1;
                        const float o0 = (float)(i0 - I.S[0]), o1 = (float)(i1 - I.S[1]);
                        const float dx = fmaxf(0.f, fmaxf(o0 * h0 - S.box[3], S.box[0] - (o0 + 1.f) * h0) - marg);
                        const float dy = fmaxf(0.f, fmaxf(o1 * h1 - S.box[4], S.box[1] - (o1 + 1.f) * h1) - marg);
                        const float d2 = fmaf(dx, dx, dy * dy);
                        if (d2 < K.rc2) {
                            const float rz = sqrtf(K.rc2 - d2) + 2.f * marg;
                            i2 = max(0, (int)floorf((S.box[2] - rz) * ih2) + I.S[2]);
                            i2b = min(nzt - 1, (int)floorf((S.box[5] + rz) * ih2) + I.S[2]);
                            row = I.cell_off + (S.ft.wx[i0] * I.nc[1] + S.ft.wy[i1]) * I.nc[2];
                        }
                    }
                    kb += 32;
                    open = true;
                }
                if (!__any_sync(kFull, i2 <= i2b)) {
                    open = false;
                    continue;
                }
                if (nseg > kSeg - 32) break;  // a round adds up to 32 segments
                int sb = 0, sn = 0, meta = 0;
                if (i2 <= i2b) {
                    const int w2 = S.ft.wz[i2];
                    const int run = min(i2b - i2 + 1, I.nc[2] - w2);
                    sb = src_start[row + w2];
                    sn = src_start[row + w2 + run] - sb;
                    meta = i0 | (i1 << 5) | (i2 << 10);
                    i2 += run;
                }
                const unsigned bal = __ballot_sync(kFull, sn > 0);
                if (sn > 0) {
                    const int pos = nseg + __popc(bal & lt);
                    S.sg_b[pos] = sb;
                    S.sg_n[pos] = sn;
                    S.sg_meta[pos] = meta;
                }
                nseg += __popc(bal);
            }
            if (nseg == 0) break;
            __syncwarp();
            stream_segments<NP>(S, I, T, K, c12, F, nseg, lane, spos_hi, spos_lo, sfrc, u_real);
            nseg = 0;
        }
        // the rest of the near queue, then the item's sums
        {
            const int nq = S.nq_n;
            __syncwarp();
            if (nq > 0) near_flush(S, T, nq, nq, lane, u_real + 3 * (size_t)F.first);
            if (lane == 0) S.nq_n = 0;
        }
        __syncwarp();
        chunk_sums(S, lane);
        if (active) {  // the item's part of the target's sum (other column groups add theirs)
            size_t o = 3 * (size_t)tidx;
#pragma unroll
            for (int c = 0; c < 3; c++)
                atomicAdd(u_real + o + c, (double)S.ks[c][lane] - (double)S.ks[3 + c][lane]);
        }
        __syncwarp();
    }
}

void launch_real_mixed(int npoly, const PbInst* inst, const PbTables* tab, const int4* items, const int* nitems_ptr,
                       int nitems_max,
                       const float4* spos_hi, const float4* spos_lo, const float4* sfrc, const int* src_start,
                       const float4* tpos_hi, const float4* tpos_lo, int ntgt_cap,
                       double* u_real, int* counter, int nsm, cudaStream_t s)
{
    if (nitems_max <= 0) return;
    cudaMemsetAsync(counter, 0, sizeof(int), s);
    cudaMemsetAsync(u_real, 0, 3 * sizeof(double) * (size_t)ntgt_cap, s);
    int blocks = nsm * 8;
    int need = (nitems_max + kRealWarps - 1) / kRealWarps;
    if (blocks > need) blocks = need;
#define PB_LAUNCH_REAL(NP)                                                                                            \
    k_real_mixed<NP><<<blocks, kRealWarps * 32, 0, s>>>(inst, tab, items, nitems_ptr, spos_hi, spos_lo, sfrc,        \
                                                         src_start, tpos_hi, tpos_lo, u_real, counter,               \
                                                         nitems_max)
    // one instantiation per even term count: a shorter Horner chain per pair
    if (npoly <= 16)
        PB_LAUNCH_REAL(16);
    else if (npoly <= 18)
        PB_LAUNCH_REAL(18);
    else if (npoly <= 20)
        PB_LAUNCH_REAL(20);
    else if (npoly <= 22)
        PB_LAUNCH_REAL(22);
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
    __shared__ double2 sh_cf[kRealWarps][kMaxCheb64];  // far-piece (T1, T2) coefficients of the current instance
    __shared__ Dbl4 sh_t[kRealWarps][32];               // the item's targets
    __shared__ float4 sh_pf[kRealWarps][32];            // staged sources rounded to FP32 (classification)
    __shared__ unsigned short sh_q[kRealWarps][1024];   // in-cutoff pairs of a chunk, target-major (t << 5 | j)
    __shared__ double sh_v[kRealWarps][3][32];          // one batch's sums per target
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nitems = min(*nitems_ptr, item_cap);
    int cur_q = -1;
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
        const DiffHConsts kd = diffh_consts(a, dd, cd);
        const DiffHConsts ke = diffh_consts(a, ee > 0 ? ee : dd, ce);  // used only when eps > 0
        const double rc2 = I.rc * I.rc;
        const double rs2 = (double)T.rs2;
        const double rf2 = T.rf2, tfs = T.tf_scale, tfo = T.tf_off;
        const int nf = T.nf;
        if (it.x != cur_q) {
            cur_q = it.x;
            __syncwarp();
            for (int k = lane; k < kMaxCheb64; k += 32) sh_cf[w][k] = make_double2(T.cf1[k], T.cf2[k]);
            __syncwarp();
        }
        ItemFrame F;
        item_frame(I, it, F);
        const bool active = lane < F.count;
        const int tidx = F.first + (active ? lane : 0);
        const int self_src = I.same ? tidx - I.tgt_off + I.src_off : -1;
        Dbl4 tp = tpos[tidx];
        if (!active) tp.x = tp.y = tp.z = 3.0e300;  // inactive lanes pair with nothing
        __syncwarp();
        sh_t[w][lane] = tp;
        // candidates are classified in FP32 against a cutoff widened by the
        // rounding of the shifted positions (|value| <= 3 L: at most 2^-24 x 3L
        // per coordinate, under 16 x 2^-24 L over a displacement vector) and of
        // the FP32 arithmetic; pairs the FP64 distance puts beyond rc add nothing
        const float tpx = (float)tp.x, tpy = (float)tp.y, tpz = (float)tp.z;
        const double lmax = fmax(I.L[0], fmax(I.L[1], I.L[2]));
        const double rcw = I.rc + 16.0 * lmax * 5.9604644775390625e-8;
        const float rcf2 = (float)(rcw * rcw * (1.0 + 1e-6));
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
                            sh_pf[w][lane] = make_float4((float)(p.x + sh0), (float)(p.y + sh1), (float)(p.z + sh2), 0.f);
                            sh_f[w][lane] = sfrc[j];
                        }
                        __syncwarp();
                        const int ncand = min(32, e - base);
                        unsigned mask = 0;
                        if (active) {
                            for (int jj = 0; jj < ncand; jj++) {
                                const float4 p = sh_pf[w][jj];
                                const float dx = tpx - p.x, dy = tpy - p.y, dz = tpz - p.z;
                                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                                mask |= (r2 < rcf2 ? 1u : 0u) << jj;
                            }
                            if (self_src >= base && self_src < base + ncand && zero_shift)
                                mask &= ~(1u << (self_src - base));
                        }
                        // compact the in-cutoff pairs target-major, then evaluate them 32 at a
                        // time with every lane busy (the FP64 pipe issues a warp instruction
                        // whatever the number of active lanes)
                        const int cnt = __popc(mask);
                        const int qoff = warp_excl_scan(cnt, lane);
                        const int total = __shfl_sync(kFull, qoff + cnt, 31);
                        for (int k = qoff; mask; k++) {
                            const int jj = __ffs(mask) - 1;
                            mask &= mask - 1;
                            sh_q[w][k] = (unsigned short)((lane << 5) | jj);
                        }
                        __syncwarp();
                        for (int qb = 0; qb < total; qb += 32) {
                            const int qi = qb + lane;
                            double c0 = 0.0, c1 = 0.0, c2 = 0.0;
                            int tq = -1;
                            if (qi < total) {
                                const int ent = sh_q[w][qi];
                                tq = ent >> 5;
                                const int jj = ent & 31;
                                const Dbl4 tt = sh_t[w][tq];
                                const Dbl4 p = sh_p[w][jj], f = sh_f[w][jj];
                                const double dx = tt.x - p.x, dy = tt.y - p.y, dz = tt.z - p.z;
                                const double r2 = dx * dx + dy * dy + dz * dz;
                                double H1 = 0.0, H2 = 0.0;
                                if (r2 >= rc2) {
                                    // beyond the cutoff in FP64 (kept by the widened FP32 test)
                                } else if (r2 < T.rtiny2 || r2 == 0.0) {
                                    if (T.blob) {
                                        series_H(T, r2, H1, H2);
                                    } else {
                                        H1 = T.self1;
                                        H2 = 0;
                                    }
                                } else if (nf > 0 && r2 >= rf2) {
                                    // far: the FP64 Chebyshev series of T1 = r H1, T2 = r^3 H2
                                    const double ir = rsqrt(r2), r = r2 * ir;
                                    const double t = fma(r, tfs, tfo), t2 = 2.0 * t;
                                    double b1x = 0.0, b1y = 0.0, b2x = 0.0, b2y = 0.0;
                                    for (int k = nf - 1; k >= 1; k--) {
                                        const double2 c = sh_cf[w][k];
                                        const double b0x = fma(t2, b1x, c.x - b2x), b0y = fma(t2, b1y, c.y - b2y);
                                        b2x = b1x;
                                        b1x = b0x;
                                        b2y = b1y;
                                        b1y = b0y;
                                    }
                                    const double2 cc = sh_cf[w][0];
                                    H1 = fma(t, b1x, cc.x - b2x) * ir;
                                    H2 = fma(t, b1y, cc.y - b2y) * (ir * ir * ir);
                                } else {
                                    const double r = sqrt(r2), ir = 1.0 / r;
                                    diffH_fast_d(r, ir, kd, H1, H2);
                                    if (T.blob && r2 < rs2) {
                                        double e1, e2;
                                        diffH_fast_d(r, ir, ke, e1, e2);
                                        H1 -= e1;
                                        H2 -= e2;
                                    }
                                }
                                const double fd = f.x * dx + f.y * dy + f.z * dz;
                                c0 = H1 * f.x + H2 * fd * dx;
                                c1 = H1 * f.y + H2 * fd * dy;
                                c2 = H1 * f.z + H2 * fd * dz;
                            }
                            // the batch is target-major: sum each target's contiguous run by a
                            // segmented scan, then its last lane hands the sum to the target's lane
#pragma unroll
                            for (int o = 1; o < 32; o <<= 1) {
                                const double u0 = __shfl_up_sync(kFull, c0, o), u1 = __shfl_up_sync(kFull, c1, o),
                                             u2 = __shfl_up_sync(kFull, c2, o);
                                const int tu = __shfl_up_sync(kFull, tq, o);
                                if (lane >= o && tu == tq) {
                                    c0 += u0;
                                    c1 += u1;
                                    c2 += u2;
                                }
                            }
                            const int tn = __shfl_down_sync(kFull, tq, 1);
                            const bool last = tq >= 0 && (lane == 31 || tn != tq);
                            if (last) {
                                sh_v[w][0][tq] = c0;
                                sh_v[w][1][tq] = c1;
                                sh_v[w][2][tq] = c2;
                            }
                            const unsigned tmask = __reduce_or_sync(kFull, last ? 1u << tq : 0u);
                            __syncwarp();
                            if ((tmask >> lane) & 1u) {
                                v0 += sh_v[w][0][lane];
                                v1 += sh_v[w][1][lane];
                                v2 += sh_v[w][2][lane];
                            }
                            __syncwarp();
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
