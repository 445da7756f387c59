// Output-stationary spreading of the FP32 grids (mixed precision): the
// Gaussian spreading of cuda/fftBrinkman.h:120-155 onto float4 grids
// (three components interleaved), organised by grid tile instead of by point.
//
// A block owns a tile of 16 x 16 x 8 grid points of one instance (fewer along
// an axis whose grid is smaller).  Each of its 256 threads owns one (x, y)
// column of the tile and keeps the column's 8 z values of the three
// components in registers.  The block enumerates the real-space cells whose
// points' windows can reach the tile (the cell list is already sorted), and
// streams those points through shared memory 256 at a time: each thread
// loads one candidate, the block keeps the points whose window meets the
// tile, and the threads lay the kept points' Gaussian weights out along the
// tile's three axes, one (point, axis) row each (zero outside the window,
// periodic wrap included).  Every column then adds f w_x w_y w_z over its 8 z values with
// packed FP32x2 FMAs; warps whose 8 x 4 column patch the window misses skip
// the point.  At the end each column is stored once: no atomics, no grid
// clear, and a fixed summation order (the result does not depend on the
// scheduling).  The window arithmetic is the FP32 one of the point-wise
// kernels (window_f32 in pb_kspace.cu): the cell of a point by a multiply
// with the inverse spacing, its offset from the window start as a
// double-float difference.
#include <algorithm>

#include "pb_device.cuh"
#include "pb_kernels.h"
#include "pb_tile.cuh"

namespace pb {

constexpr int kTile = 16;            // tile edge along x and y (grid points)
constexpr int kTileZ = 8;            // tile edge along z (the registers a column holds)
constexpr int kSpreadThreads = 256;  // one per (x, y) column of the tile
constexpr int kSegRound = 256;       // cell columns enumerated per round (one per thread)
constexpr int kWts = 2 * kTile + kTileZ;  // tile-aligned weights of a point: x, y, z

struct SpreadSmem {
    float w[kSpreadThreads][kWts];    // tile-aligned weights of the kept points (x: 0..15, y: 16..31, z: 32..39)
    float4 f[kSpreadThreads];         // forces of the kept points
    unsigned mask[kSpreadThreads];    // the warps (8 x 4 column patches) whose columns a kept point's window meets
    int j[kSpreadThreads];            // sorted index of a kept point
    short g0[kSpreadThreads][3];      // window start per axis (|start| < 1024)
    float base[kSpreadThreads][3];    // offset of the point from its window start
    int seg_b[2 * kSegRound];         // point segments of the round: first index
    int seg_pre[2 * kSegRound + 1];   // exclusive prefix of the segment lengths
    int wsum[kSpreadThreads / 32 + 1];
};

__global__ void __launch_bounds__(kSpreadThreads, 4)  // 64 registers; 3 blocks per SM (80) measured 9% slower
    k_spread_tile(const PbInst* __restrict__ inst, const int* __restrict__ bucket_inst, int ntx, int nty, int ntz,
                  const int* __restrict__ src_start, const float4* __restrict__ pa, const float4* __restrict__ pb,
                  const float4* __restrict__ frc, float* __restrict__ grid)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SpreadSmem& S = *reinterpret_cast<SpreadSmem*>(smem_raw);
    const int tpi = ntx * nty * ntz;
    const int qi = blockIdx.x / tpi, tile = blockIdx.x - qi * tpi;
    const PbInst& I = inst[bucket_inst[qi]];
    if (I.n_src <= 0 || I.n_tgt <= 0) return;  // the FFT passes and the gather skip this grid too
    const int tx = tile % ntx, ty = (tile / ntx) % nty, tz = tile / (ntx * nty);
    const int T[3] = {min(kTile, I.M[0]), min(kTile, I.M[1]), min(kTileZ, I.M[2])};
    const int t0[3] = {tx * T[0], ty * T[1], tz * T[2]};
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    // column of this thread: warp w holds the 8 x 4 patch at x 8 (w & 1), y 4 (w >> 1)
    const int cx = ((w & 1) << 3) + (lane & 7), cy = ((w >> 1) << 2) + (lane >> 3);
    const bool owner = cx < T[0] && cy < T[1];
    float2 ax[kTileZ / 2], ay[kTileZ / 2], az[kTileZ / 2];
#pragma unroll
    for (int k = 0; k < kTileZ / 2; k++) ax[k] = ay[k] = az[k] = make_float2(0.f, 0.f);

    int fx, nx, fy, ny, fz, nz;
    cell_range(I, 0, t0[0], T[0], fx, nx);
    cell_range(I, 1, t0[1], T[1], fy, ny);
    cell_range(I, 2, t0[2], T[2], fz, nz);
    const int npairs = nx * ny;
    const float inv_eta = I.inv_eta_f;
    for (int rb = 0; rb < npairs; rb += kSegRound) {
        // the round's cell columns (one per thread), each a z-run of cells cut at the periodic wrap
        int b0 = 0, n0 = 0, b1 = 0, n1 = 0;
        {
            const int pr = rb + tid;
            if (pr < npairs) {
                const int ix = pr % nx, iy = pr / nx;
                const int row = I.cell_off + (pmod(fx + ix, I.nc[0]) * I.nc[1] + pmod(fy + iy, I.nc[1])) * I.nc[2];
                const int z0 = pmod(fz, I.nc[2]);
                const int run0 = min(nz, I.nc[2] - z0);
                b0 = src_start[row + z0];
                n0 = src_start[row + z0 + run0] - b0;
                if (run0 < nz) {
                    b1 = src_start[row];
                    n1 = src_start[row + nz - run0] - b1;
                }
            }
        }
        int nseg;
        const int sidx = block_scan256((n0 > 0) + (n1 > 0), S.wsum, &nseg);
        {
            int k = sidx;
            if (n0 > 0) {
                S.seg_b[k] = b0;
                S.seg_pre[k++] = n0;  // lengths for now
            }
            if (n1 > 0) {
                S.seg_b[k] = b1;
                S.seg_pre[k] = n1;
            }
        }
        __syncthreads();
        // exclusive prefix of the segment lengths (two segments per thread)
        int npts;
        {
            const int a = 2 * tid, b = 2 * tid + 1;
            const int la = a < nseg ? S.seg_pre[a] : 0, lb = b < nseg ? S.seg_pre[b] : 0;
            const int ex = block_scan256(la + lb, S.wsum, &npts);
            __syncthreads();
            if (a < nseg) S.seg_pre[a] = ex;
            if (b < nseg) S.seg_pre[b] = ex + la;
            if (tid == 0) S.seg_pre[nseg] = npts;
            __syncthreads();
        }
        for (int cb = 0; cb < npts; cb += kSpreadThreads) {
            // 1. a candidate per thread: its window start on each axis and whether it meets the tile
            const int p = cb + tid;
            bool keep = false;
            int jj = 0, g0[3] = {0, 0, 0};
            float bs[3] = {0.f, 0.f, 0.f};
            if (p < npts) {
                int lo = 0, hi = nseg - 1;  // last segment starting at or before p
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (S.seg_pre[mid] <= p)
                        lo = mid;
                    else
                        hi = mid - 1;
                }
                jj = S.seg_b[lo] + (p - S.seg_pre[lo]);
                const float4 h4 = pa[jj], l4 = pb[jj];
                const float xh[3] = {h4.x, h4.y, h4.z}, xl[3] = {l4.x, l4.y, l4.z};
                keep = true;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    const float gi = I.gihf[a];
                    const int c = min(max((int)floorf(fmaf(xh[a], gi, xl[a] * gi)), 0), I.M[a] - 1);
                    g0[a] = c - I.Pa[a] / 2 + 1;
                    const float gf = (float)g0[a], hh = I.ghh[a];
                    const float pr = gf * hh, er = fmaf(gf, hh, -pr);  // g0 hh = pr + er exactly
                    bs[a] = ((xh[a] - pr) - er) + (xl[a] - gf * I.ghl[a]);
                    // the window covers (g0 + k) mod M, k < P, the tile [t0, t0 + T): two arcs
                    // of the periodic axis meet iff the start of one lies in the other
                    const int rel = (t0[a] - g0[a]) & (I.M[a] - 1);  // tile start in the window's frame
                    const int st = (g0[a] - t0[a]) & (I.M[a] - 1);   // window start in the tile's frame
                    keep = keep && (rel < I.Pa[a] || st < T[a]);
                }
            }
            // 2. keep the candidates that meet the tile, in candidate order
            int K;
            const int slot = block_scan256(keep ? 1 : 0, S.wsum, &K);
            if (keep) {
                S.j[slot] = jj;
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    S.g0[slot][a] = g0[a];
                    S.base[slot][a] = bs[a];
                }
            }
            __syncthreads();
            // 3a. thread t: kept point t's force and the warps whose patch its window meets
            if (tid < K) {
                S.f[tid] = frc[S.j[tid]];
                unsigned occ[2] = {0u, 0u};  // tile positions (x, y) inside the window
#pragma unroll
                for (int a = 0; a < 2; a++) {
                    const int o0 = (t0[a] - S.g0[tid][a]) & (I.M[a] - 1);
#pragma unroll
                    for (int k = 0; k < kTile; k++)
                        if (k < T[a] && ((o0 + k) & (I.M[a] - 1)) < I.Pa[a]) occ[a] |= 1u << k;
                }
                unsigned m = 0;
#pragma unroll
                for (int ww = 0; ww < kSpreadThreads / 32; ww++)
                    if (((occ[0] >> ((ww & 1) << 3)) & 0xffu) && ((occ[1] >> ((ww >> 1) << 2)) & 0xfu)) m |= 1u << ww;
                S.mask[tid] = m;
            }
            // 3b. all threads, one (point, axis) row each: the K x 40 tile-aligned weights
            // along the row, zero outside the window
            for (int e = tid; e < 3 * K; e += kSpreadThreads) {
                const int q = e / 3, a = e - 3 * q;
                // per-axis values by selection (a runtime index would put the arrays in local memory)
                const int ta = a == 0 ? t0[0] : a == 1 ? t0[1] : t0[2];
                const int Ta = a == 0 ? T[0] : a == 1 ? T[1] : T[2];
                const int nk = a == 2 ? kTileZ : kTile, Mm = I.M[a] - 1, P = I.Pa[a];
                const float hh = I.ghh[a], b = S.base[q][a];
                float* row = &S.w[q][a * kTile];
                int o = (ta - S.g0[q][a]) & Mm;  // window offset of the tile's first point on this axis
                for (int k = 0; k < nk; k++, o = (o + 1) & Mm) {
                    const float dx = fmaf(-(float)o, hh, b);
                    row[k] = (k < Ta && o < P) ? expf(-dx * dx * inv_eta) : 0.f;
                }
            }
            __syncthreads();
            // 4. warp w adds the kept points whose window meets its patch, two at a time
            for (int qb = 0; qb < K; qb += 32) {
                unsigned m = __ballot_sync(kFull, qb + lane < K && ((S.mask[qb + lane] >> w) & 1u));
                while (m) {
                    const int q0 = qb + __ffs(m) - 1;
                    m &= m - 1;
                    const int q1 = m ? qb + __ffs(m) - 1 : q0;
                    const float s1 = m ? 1.f : 0.f;  // the second point's share (none when the list is odd)
                    if (m) m &= m - 1;
                    const float w0 = S.w[q0][cx] * S.w[q0][kTile + cy];
                    const float w1 = S.w[q1][cx] * S.w[q1][kTile + cy] * s1;
                    const float4 f0 = S.f[q0], f1 = S.f[q1];
                    const float4* z0 = reinterpret_cast<const float4*>(&S.w[q0][2 * kTile]);
                    const float4* z1 = reinterpret_cast<const float4*>(&S.w[q1][2 * kTile]);
                    const float2 a0 = make_float2(f0.x * w0, f0.x * w0), b0 = make_float2(f0.y * w0, f0.y * w0),
                                 c0 = make_float2(f0.z * w0, f0.z * w0);
                    const float2 a1 = make_float2(f1.x * w1, f1.x * w1), b1 = make_float2(f1.y * w1, f1.y * w1),
                                 c1 = make_float2(f1.z * w1, f1.z * w1);
#pragma unroll
                    for (int k = 0; k < kTileZ / 4; k++) {
                        const float4 u = z0[k], v = z1[k];
                        const float2 ul = make_float2(u.x, u.y), uh = make_float2(u.z, u.w);
                        const float2 vl = make_float2(v.x, v.y), vh = make_float2(v.z, v.w);
                        ax[2 * k] = __ffma2_rn(a1, vl, __ffma2_rn(a0, ul, ax[2 * k]));
                        ax[2 * k + 1] = __ffma2_rn(a1, vh, __ffma2_rn(a0, uh, ax[2 * k + 1]));
                        ay[2 * k] = __ffma2_rn(b1, vl, __ffma2_rn(b0, ul, ay[2 * k]));
                        ay[2 * k + 1] = __ffma2_rn(b1, vh, __ffma2_rn(b0, uh, ay[2 * k + 1]));
                        az[2 * k] = __ffma2_rn(c1, vl, __ffma2_rn(c0, ul, az[2 * k]));
                        az[2 * k + 1] = __ffma2_rn(c1, vh, __ffma2_rn(c0, uh, az[2 * k + 1]));
                    }
                }
            }
            __syncthreads();
        }
    }
    if (!owner) return;
    float4* g4 = reinterpret_cast<float4*>(grid + I.grid_off) +
                 ((size_t)(t0[0] + cx) * I.M[1] + (t0[1] + cy)) * I.M[2] + t0[2];
#pragma unroll
    for (int k = 0; k < kTileZ / 2; k++) {
        if (2 * k < T[2]) g4[2 * k] = make_float4(ax[k].x, ay[k].x, az[k].x, 0.f);
        if (2 * k + 1 < T[2]) g4[2 * k + 1] = make_float4(ax[k].y, ay[k].y, az[k].y, 0.f);
    }
}

size_t spread_tile_smem() { return sizeof(SpreadSmem); }

void launch_spread_tiles(const PbInst* inst, const int* bucket_inst, int nb, const int* M, const int* src_start,
                         const float4* pos_a, const float4* pos_b, const float4* frc, float* grid, cudaStream_t s)
{
    if (nb <= 0) return;
    const int ntx = M[0] / std::min(kTile, M[0]), nty = M[1] / std::min(kTile, M[1]),
              ntz = M[2] / std::min(kTileZ, M[2]);
    const long long blocks = (long long)nb * ntx * nty * ntz;
    const int smem = (int)sizeof(SpreadSmem);
    cudaFuncSetAttribute(k_spread_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    k_spread_tile<<<(unsigned)blocks, kSpreadThreads, smem, s>>>(inst, bucket_inst, ntx, nty, ntz, src_start, pos_a,
                                                                   pos_b, frc, grid);
}

}  // namespace pb
