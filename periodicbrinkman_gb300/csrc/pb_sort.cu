// Cell binning, counting sort, sorted particle records and work-item
// construction for the real-space sum and the tiled spreading (device-built
// cell lists over all instances of a batch).
#include "pb_device.cuh"
#include "pb_kernels.h"

namespace pb {

// A non-finite coordinate is binned as 0 and flags its instance in bad[q].
__device__ __forceinline__ double finite_or_flag(double v, int* bad, int q)
{
    if (isfinite(v)) return v;
    if (bad) bad[q] = 1;
    return 0.0;
}

// Block-wide exclusive prefix sum (all threads of the block take part).
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums)
{
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int w = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(kFull, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    int base = wid > 0 ? warp_sums[wid - 1] : 0;
    return base + x - v;
}

__global__ void k_prepare_mixed(const double* __restrict__ pos, const double* __restrict__ frc,
                                const int* __restrict__ perm, const int* __restrict__ offsets,
                                const PbInst* __restrict__ inst, int ninst, float4* __restrict__ pos_hi,
                                float4* __restrict__ pos_lo, float4* __restrict__ frc_out, int* __restrict__ bad)
{
    int sidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (sidx >= offsets[ninst]) return;
    int p = perm[sidx];
    int q = find_instance(offsets, ninst, p);
    const PbInst& I = inst[q];
    float hi[3], lo[3];
#pragma unroll
    for (int a = 0; a < 3; a++)
        split_double(wrap_coord_r(finite_or_flag(pos[3 * (size_t)p + a], bad, q), I.L[a], I.iL[a]), hi[a], lo[a]);
    pos_hi[sidx] = make_float4(hi[0], hi[1], hi[2], __int_as_float(q));
    pos_lo[sidx] = make_float4(lo[0], lo[1], lo[2], 0.f);
    if (frc)
        frc_out[sidx] = make_float4((float)finite_or_flag(frc[3 * (size_t)p], bad, q),
                                    (float)finite_or_flag(frc[3 * (size_t)p + 1], bad, q),
                                    (float)finite_or_flag(frc[3 * (size_t)p + 2], bad, q), 0.f);
}

void launch_prepare_mixed(const double* pos, const double* frc, const int* perm, int ncap, const int* offsets,
                          const PbInst* inst, int ninst, float4* pos_hi, float4* pos_lo, float4* frc_out, int* bad,
                          cudaStream_t s)
{
    if (ncap <= 0) return;
    k_prepare_mixed<<<(ncap + 255) / 256, 256, 0, s>>>(pos, frc, perm, offsets, inst, ninst, pos_hi, pos_lo,
                                                        frc_out, bad);
}

__global__ void k_prepare_fp64(const double* __restrict__ pos, const double* __restrict__ frc,
                               const int* __restrict__ perm, const int* __restrict__ offsets,
                               const PbInst* __restrict__ inst, int ninst, Dbl4* __restrict__ pos_out,
                               Dbl4* __restrict__ frc_out, int* __restrict__ bad)
{
    int sidx = blockIdx.x * blockDim.x + threadIdx.x;
    if (sidx >= offsets[ninst]) return;
    int p = perm[sidx];
    int q = find_instance(offsets, ninst, p);
    const PbInst& I = inst[q];
    double w[3];
#pragma unroll
    for (int a = 0; a < 3; a++) w[a] = wrap_coord_r(finite_or_flag(pos[3 * (size_t)p + a], bad, q), I.L[a], I.iL[a]);
    pos_out[sidx] = make_dbl4(w[0], w[1], w[2], (double)q);
    if (frc)
        frc_out[sidx] = make_dbl4(finite_or_flag(frc[3 * (size_t)p], bad, q),
                                  finite_or_flag(frc[3 * (size_t)p + 1], bad, q),
                                  finite_or_flag(frc[3 * (size_t)p + 2], bad, q), 0.0);
}

void launch_prepare_fp64(const double* pos, const double* frc, const int* perm, int ncap, const int* offsets,
                         const PbInst* inst, int ninst, Dbl4* pos_out, Dbl4* frc_out, int* bad, cudaStream_t s)
{
    if (ncap <= 0) return;
    k_prepare_fp64<<<(ncap + 255) / 256, 256, 0, s>>>(pos, frc, perm, offsets, inst, ninst, pos_out, frc_out,
                                                       bad);
}

// Work items of the real-space kernel: each cell row (c0, c1) of an instance
// is walked along z and cut into row items of 32 consecutive targets (cells
// may be split between items, so warps stay full), fewer where the row ends
// or where 32 targets would span more than the instance's zspan cells (sparse targets,
// such as a target set half the size of the sources, fill a warp only over
// many cells: a longer item costs more candidates per item but fewer per
// target, and every lane then holds one).  Each row item becomes
// `G` = csplit work items, one per group of stencil columns, so that small
// instances still fill the GPU.  One thread per row start: a counting walk,
// then the emitting walk into its range.  A row gives at most
// targets/32 + cells items.
// Item = {instance, first target, local row, count | za << 8 | zb << 16 | group << 24}.
template <bool EMIT>
__device__ void walk_row(const int* __restrict__ start, int row0, int nz, int q, int rowl, int G, int zspan,
                         int4* items, int k0, int cap, int& nitems)
{
    int k = 0, z = 0;
    int t = start[row0];
    const int end = start[row0 + nz];
    while (t < end) {
        while (start[row0 + z + 1] <= t) z++;  // za: the cell of target t
        const int za = z;
        const int lim = min(min(t + 32, end), start[row0 + min(za + zspan, nz)]);
        while (start[row0 + z + 1] <= lim - 1) z++;  // zb: the cell of target lim - 1
        for (int g = 0; g < G; g++, k++)
            if (EMIT && k0 + k < cap)
                items[k0 + k] = make_int4(q, t, rowl, (lim - t) | (za << 8) | (z << 16) | (g << 24));
        t = lim;
    }
    nitems = k;
}

// Row items of every row start cell: a warp looks at 32 cells at a time, and
// for each row start among them stages the row's cell starts in shared memory
// (coalesced) and lets one lane walk the row there (the walk's dependent
// loads then cost shared-memory latency); each row reserves its range of the
// item array with one atomic.
constexpr int kItemWarps = 8;

__global__ void __launch_bounds__(kItemWarps * 32)
    k_build_items(const int* __restrict__ start, const int* __restrict__ cell_offsets,
                  const PbInst* __restrict__ inst, int ninst, int4* __restrict__ items, int cap,
                  int* __restrict__ nitems, int* __restrict__ status)
{
    __shared__ int st[kItemWarps][129];  // nc[2] <= 128
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ncell = cell_offsets[ninst];
    const int nwarps = gridDim.x * kItemWarps;
    for (int cb = (blockIdx.x * kItemWarps + w) * 32; cb < ncell; cb += nwarps * 32) {
        const int c = cb + lane;
        int q = 0, local = 0;
        bool rs = false;
        if (c < ncell) {
            q = find_instance(cell_offsets, ninst, c);
            local = c - inst[q].cell_off;
            rs = local < inst[q].ncell && local % inst[q].nc[2] == 0;
        }
        unsigned m = __ballot_sync(kFull, rs);
        while (m) {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const int rc = __shfl_sync(kFull, c, src), rq = __shfl_sync(kFull, q, src),
                      rl = __shfl_sync(kFull, local, src);
            const PbInst& I = inst[rq];
            const int nz = I.nc[2];
            __syncwarp();
            for (int z = lane; z <= nz; z += 32) st[w][z] = start[rc + z];
            __syncwarp();
            if (lane == 0) {
                const int G = max(1, I.csplit), zspan = min(max(I.zspan, 1), kItemCells);
                int n = 0;
                walk_row<false>(st[w], 0, nz, rq, rl / nz, G, zspan, nullptr, 0, 0, n);
                if (n > 0) {
                    const int k0 = atomicAdd(nitems, n);
                    if (k0 + n > cap) atomicOr(status, kCapItems);  // items dropped: reported, not silent
                    walk_row<true>(st[w], 0, nz, rq, rl / nz, G, zspan, items, k0, cap, n);
                }
            }
        }
    }
}

void launch_build_items(const int* start, int ncell_cap, const int* cell_offsets, const PbInst* inst, int ninst,
                        int4* items, int cap, int* nitems, int* status, int nsm, cudaStream_t s)
{
    cudaMemsetAsync(nitems, 0, sizeof(int), s);
    if (ncell_cap <= 0) return;
    long long blocks = ((long long)ncell_cap + 32 * kItemWarps - 1) / (32 * kItemWarps);
    if (blocks > (long long)nsm * 8) blocks = (long long)nsm * 8;
    k_build_items<<<(int)blocks, kItemWarps * 32, 0, s>>>(start, cell_offsets, inst, ninst, items, cap, nitems,
                                                          status);
}

// ---- cell lists of sources and targets, four launches for both ----
// Particle side: index p < ncap_s is source p, p >= ncap_s is target p - ncap_s.
// The counts of the two sets are cstride apart, as are their starts.
constexpr int kCellScanThreads = 1024;
constexpr int kCellScanTile = 4 * kCellScanThreads;  // counts per scan block (four per thread)
constexpr unsigned long long kFlagAgg = 1ull << 62, kFlagPrefix = 2ull << 62;
constexpr int kScanSpinLimit = 1 << 22;  // look-back waits (with back-off) before a block gives up
constexpr int kSortMax = 1024;           // larger cells keep the scatter order

int cell_list_stride(int ncell_cap) { return (ncell_cap + 1 + 3) & ~3; }

static int cell_scan_tiles(int ncell_cap) { return (cell_list_stride(ncell_cap) + kCellScanTile - 1) / kCellScanTile; }

// counts [2][cstride], two tickets (+ padding to 16 bytes), look-back flags [2][tiles]
size_t cell_list_zero_bytes(int ncell_cap)
{
    return sizeof(int) * (2 * (size_t)cell_list_stride(ncell_cap) + 4) +
           sizeof(unsigned long long) * 2 * (size_t)cell_scan_tiles(ncell_cap);
}

// Position of target t of instance q: its own targets (y) or its sources (x).
__device__ __forceinline__ const double* cl_target(const CellListArgs& A, int q, int t)
{
    const int yo = A.y_off[q], local = t - A.tgt_off[q];
    return yo >= 0 ? A.y + 3 * (size_t)(yo + local) : A.x + 3 * (size_t)(A.src_off[q] + local);
}

// wrap_coord_r without its FP64 arithmetic for a coordinate already inside
// [0, L) by more than a few ulps (the usual case; compared as bit patterns,
// which order non-negative doubles): there wrap_coord_r returns v itself.
__device__ __forceinline__ double wrap_in_box(double v, double L, double iL)
{
    const long long vb = __double_as_longlong(v), lb = __double_as_longlong(L);
    if (vb >= 0 && vb < lb - 8) return v;
    return wrap_coord_r(v, L, iL);
}

// FP32 sort key of a particle within its cell: z wrapped in FP32.
__device__ __forceinline__ float cl_zkey(const PbInst& I, double z64)
{
    const float Lz = (float)I.L[2], iLz = (float)I.iL[2];
    float z = (float)z64;
    z -= Lz * floorf(z * iLz);
    return (z == z) ? z : 0.f;
}

// Per particle: its cell, its arrival slot in the cell, its instance and its
// z key (key = {cell, slot, instance, z bits}).
__global__ void k_bin_cells(CellListArgs A)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.ncap_s + A.ncap_t) return;  // (with no target set, tgt_off counts the sources)
    const bool tgt = p >= A.ncap_s;
    const int i = tgt ? p - A.ncap_s : p;
    const int* off = tgt ? A.tgt_off : A.src_off;
    if (i >= off[A.ninst]) return;
    const int q = find_instance(off, A.ninst, i);
    const PbInst& I = A.inst[q];
    const double* pos = tgt ? cl_target(A, q, i) : A.x + 3 * (size_t)i;
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const double w = wrap_in_box(finite_or_flag(pos[a], A.bad, q), I.L[a], I.iL[a]);
        const int ci = (int)(w * I.ih[a]);
        c[a] = ci >= I.nc[a] ? I.nc[a] - 1 : ci;
    }
    const int g = I.cell_off + (c[0] * I.nc[1] + c[1]) * I.nc[2] + c[2];
    const int slot = atomicAdd(&A.zero[(tgt ? A.cstride : 0) + g], 1);
    (tgt ? A.key_t : A.key_s)[i] = make_int4(g, slot, q, __float_as_int(cl_zkey(I, pos[2])));
}

// Exclusive scan of the counts [0, n_act] of each set (the entry at n_act is
// zero and receives the total), single pass: blocks take tiles in the order
// they start (a ticket per set), publish their tile's sum, and add the sums
// of the tiles before theirs by looking back until a tile with its inclusive
// prefix published.  A block waits only on tiles whose blocks started before
// it, so every wait ends; each wait is bounded all the same (kScanStall).
__global__ void __launch_bounds__(kCellScanThreads) k_scan_cells(CellListArgs A, int nsets)
{
    __shared__ int ws[32];
    __shared__ int s_ticket, s_prefix;
    const int cstride = A.cstride, ntiles = A.ntiles;
    int* tickets = A.zero + 2 * cstride;
    unsigned long long* flags = reinterpret_cast<unsigned long long*>(tickets + 4);
    const int set = nsets == 2 ? (int)(blockIdx.x & 1) : 0;
    if (threadIdx.x == 0) s_ticket = atomicAdd(&tickets[set], 1);
    __syncthreads();
    const int tile = s_ticket;
    const int n = A.cell_off[A.ninst] + 1;
    const int base = tile * kCellScanTile;
    if (tile >= ntiles || base >= n) return;
    const int* cnt = A.zero + set * cstride;
    int* out = A.start + set * cstride;
    unsigned long long* fl = flags + (size_t)set * ntiles;
    const int i0 = base + 4 * threadIdx.x;
    int4 v = make_int4(0, 0, 0, 0);
    if (i0 < n) v = *reinterpret_cast<const int4*>(cnt + i0);  // cstride is a multiple of 4: in bounds
    const int sum = v.x + v.y + v.z + v.w;
    const int ex = block_exclusive_scan(sum, ws);
    if (threadIdx.x == kCellScanThreads - 1) {
        const int total = ex + sum;
        if (tile == 0) {
            atomicExch(&fl[0], kFlagPrefix | (unsigned)total);
            s_prefix = 0;
        } else {
            atomicExch(&fl[tile], kFlagAgg | (unsigned)total);
            int prefix = 0, j = tile - 1, spins = 0;
            while (j >= 0) {
                const unsigned long long w = atomicAdd(&fl[j], 0ull);
                if ((w >> 62) == 0) {
                    if (++spins > kScanSpinLimit) {
                        atomicOr(&A.bad[A.ninst], kScanStall);
                        break;
                    }
                    __nanosleep(spins < 64 ? 32 : 256);
                    continue;
                }
                prefix += (int)(unsigned)(w & 0xffffffffu);
                if ((w >> 62) == 2) break;
                j--;
            }
            atomicExch(&fl[tile], kFlagPrefix | (unsigned)(prefix + total));
            s_prefix = prefix;
        }
    }
    __syncthreads();
    const int e = s_prefix + ex;
    const int r[4] = {e, e + v.x, e + v.x + v.y, e + v.x + v.y + v.z};
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (i0 + k < n) out[i0 + k] = r[k];
}

// Each cell's entries {particle, z bits} in arrival order.
__global__ void k_scatter_cells(CellListArgs A)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.ncap_s + A.ncap_t) return;
    const bool tgt = p >= A.ncap_s;
    const int i = tgt ? p - A.ncap_s : p;
    if (i >= (tgt ? A.tgt_off : A.src_off)[A.ninst]) return;
    const int4 k = (tgt ? A.key_t : A.key_s)[i];
    const int* start = A.start + (tgt ? A.cstride : 0);
    (tgt ? A.perm_tmp_t : A.perm_tmp_s)[start[k.x] + k.y] = make_int2(i, k.w);
}

// The sorted record of particle v of instance q at position `slot` of its list.
template <bool MIXED>
__device__ __forceinline__ void cl_record(const CellListArgs& A, bool tgt, int q, int v, const double* pos, int slot)
{
    const PbInst& I = A.inst[q];
    double w[3];
#pragma unroll
    for (int a = 0; a < 3; a++) w[a] = wrap_in_box(finite_or_flag(pos[a], A.bad, q), I.L[a], I.iL[a]);
    const double* fr = tgt ? nullptr : A.f + 3 * (size_t)v;
    if constexpr (MIXED) {
        float hi[3], lo[3];
#pragma unroll
        for (int a = 0; a < 3; a++) split_double(w[a], hi[a], lo[a]);
        float4* ph = (float4*)(tgt ? A.tpos_a : A.spos_a);
        float4* pl = (float4*)(tgt ? A.tpos_b : A.spos_b);
        ph[slot] = make_float4(hi[0], hi[1], hi[2], __int_as_float(q));
        pl[slot] = make_float4(lo[0], lo[1], lo[2], 0.f);
        if (fr)
            ((float4*)A.sfrc)[slot] = make_float4((float)finite_or_flag(fr[0], A.bad, q),
                                                  (float)finite_or_flag(fr[1], A.bad, q),
                                                  (float)finite_or_flag(fr[2], A.bad, q), 0.f);
    } else {
        ((Dbl4*)(tgt ? A.tpos_a : A.spos_a))[slot] = make_dbl4(w[0], w[1], w[2], (double)q);
        if (fr)
            ((Dbl4*)A.sfrc)[slot] = make_dbl4(finite_or_flag(fr[0], A.bad, q), finite_or_flag(fr[1], A.bad, q),
                                              finite_or_flag(fr[2], A.bad, q), 0.0);
    }
}

// Sort of every cell by (z wrapped in FP32, index), a thread per particle,
// fused with the writing of the sorted records: particle v goes to slot
// start + #{u in cell : (z_u, u) < (z_v, v)}, counted over the cell's entries
// (contiguous, so the threads of a cell read the same few lines).  Consecutive
// targets then lie close in z (narrower real-space work items) and the order,
// hence every summation order downstream, does not depend on the scatter's
// atomics.  Cells of more than kSortMax entries keep the scatter order.
template <bool MIXED>
__global__ void k_sort_prepare(CellListArgs A)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= A.ncap_s + A.ncap_t) return;
    const bool tgt = p >= A.ncap_s;
    const int v = tgt ? p - A.ncap_s : p;
    if (v >= (tgt ? A.tgt_off : A.src_off)[A.ninst]) return;
    const int4 k = (tgt ? A.key_t : A.key_s)[v];
    const int q = k.z;
    const double* pos = tgt ? cl_target(A, q, v) : A.x + 3 * (size_t)v;
    const int* start = A.start + (tgt ? A.cstride : 0);
    const int b = start[k.x], n = start[k.x + 1] - b;
    int rank = k.y;
    if (n <= kSortMax) {
        const int2* ent = (tgt ? A.perm_tmp_t : A.perm_tmp_s) + b;
        const float z = __int_as_float(k.w);
        rank = 0;
        for (int j = 0; j < n; j++) {
            const int2 u = ent[j];
            const float zu = __int_as_float(u.y);
            rank += (zu < z) || (zu == z && u.x < v);
        }
        rank = min(rank, max(n - 1, 0));  // (stale entries after a scan that gave up: stay in the cell)
    }
    (tgt ? A.perm_t : A.perm_s)[b + rank] = v;
    cl_record<MIXED>(A, tgt, q, v, pos, b + rank);
}

void launch_cell_lists(const CellListArgs& args, bool mixed, int nsm, cudaStream_t s)
{
    CellListArgs a = args;
    a.cstride = cell_list_stride(a.ncell_cap);
    a.ntiles = cell_scan_tiles(a.ncell_cap);
    const int nsets = a.two ? 2 : 1;
    if (!a.two) a.ncap_t = 0;
    if (a.ncell_cap <= 0) return;
    const long long np = (long long)a.ncap_s + a.ncap_t;
    const unsigned pblocks = (unsigned)((np + 255) / 256);
    if (np > 0) k_bin_cells<<<pblocks, 256, 0, s>>>(a);
    k_scan_cells<<<(unsigned)(nsets * a.ntiles), kCellScanThreads, 0, s>>>(a, nsets);  // empty sets get zero starts
    if (np > 0) k_scatter_cells<<<pblocks, 256, 0, s>>>(a);
    if (np > 0 && mixed) k_sort_prepare<true><<<pblocks, 256, 0, s>>>(a);
    if (np > 0 && !mixed) k_sort_prepare<false><<<pblocks, 256, 0, s>>>(a);
}

}  // namespace pb
