// Cell binning, counting sort and work-item construction for the real-space
// sum (device-built cell list over all instances of a batch).
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

__global__ void k_bin(const double* __restrict__ pos, const int* __restrict__ offsets,
                      const PbInst* __restrict__ inst, int ninst, int* __restrict__ cell_of, int* __restrict__ counts,
                      int* __restrict__ bad)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= offsets[ninst]) return;
    int q = find_instance(offsets, ninst, p);
    const PbInst& I = inst[q];
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        double w = wrap_coord_r(finite_or_flag(pos[3 * (size_t)p + a], bad, q), I.L[a], I.iL[a]);
        int ci = (int)(w * I.ih[a]);
        c[a] = ci >= I.nc[a] ? I.nc[a] - 1 : ci;
    }
    int g = I.cell_off + (c[0] * I.nc[1] + c[1]) * I.nc[2] + c[2];
    cell_of[p] = g;
    atomicAdd(&counts[g], 1);
}

void launch_bin(const double* pos, int ncap, const int* offsets, const PbInst* inst, int ninst, int* cell_of,
                int* counts, int* bad, cudaStream_t s)
{
    if (ncap <= 0) return;
    k_bin<<<(ncap + 255) / 256, 256, 0, s>>>(pos, offsets, inst, ninst, cell_of, counts, bad);
}

// ---- exclusive scan (reduce-then-scan, recursive over block sums) ----
constexpr int kScanBlock = 1024;

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

// n_act (optional): entries at and beyond *n_act are zero and their outputs are
// not needed past index *n_act, so blocks that start beyond it only report 0.
__global__ void k_scan_blocks(const int* __restrict__ in, int* __restrict__ out, int n, int* __restrict__ block_sums,
                              const int* __restrict__ n_act)
{
    __shared__ int ws[32];
    if (n_act && blockIdx.x * kScanBlock > *n_act) {
        if (threadIdx.x == 0) block_sums[blockIdx.x] = 0;
        return;
    }
    int i = blockIdx.x * kScanBlock + threadIdx.x;
    int v = i < n ? in[i] : 0;
    int ex = block_exclusive_scan(v, ws);
    if (i < n) out[i] = ex;
    if (threadIdx.x == blockDim.x - 1) block_sums[blockIdx.x] = ex + v;
}

__global__ void k_scan_add(int* __restrict__ out, int n, const int* __restrict__ block_offsets,
                           const int* __restrict__ n_act)
{
    if (n_act && blockIdx.x * kScanBlock > *n_act) return;
    int i = blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += block_offsets[blockIdx.x];
}

__global__ void k_set_total(int* out, int n, const int* in, const int* n_act)
{
    // out[n] = out[n-1] + in[n-1] (with fewer actual entries, out[n_act] is the total already)
    if (n_act && *n_act < n) return;
    out[n] = (n > 0) ? out[n - 1] + in[n - 1] : 0;
}

size_t scan_tmp_ints(int n)
{
    size_t total = 0;
    int m = n;
    while (m > 1) {
        int nb = (m + kScanBlock - 1) / kScanBlock;
        total += 2 * (size_t)nb + 2;
        m = nb;
    }
    return total + 4;
}

static void scan_rec(const int* in, int* out, int n, int* tmp, const int* n_act, cudaStream_t s)
{
    int nb = (n + kScanBlock - 1) / kScanBlock;
    int* sums = tmp;
    int* sums_scan = tmp + nb + 1;
    k_scan_blocks<<<nb, kScanBlock, 0, s>>>(in, out, n, sums, n_act);
    if (nb > 1) {
        scan_rec(sums, sums_scan, nb, tmp + 2 * (size_t)nb + 2, nullptr, s);
        k_scan_add<<<nb, kScanBlock, 0, s>>>(out, n, sums_scan, n_act);
    }
}

void launch_exclusive_scan(const int* in, int* out, int n, int* tmp, cudaStream_t s, const int* n_act)
{
    if (n <= 0) {
        cudaMemsetAsync(out, 0, sizeof(int), s);
        return;
    }
    scan_rec(in, out, n, tmp, n_act, s);
    k_set_total<<<1, 1, 0, s>>>(out, n, in, n_act);
}

__global__ void k_scatter(const int* __restrict__ cell_of, const int* __restrict__ ntot, const int* __restrict__ start,
                          int* __restrict__ fill, int* __restrict__ perm)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= *ntot) return;
    int c = cell_of[p];
    int slot = start[c] + atomicAdd(&fill[c], 1);
    perm[slot] = p;
}

void launch_scatter(const int* cell_of, int ncap, const int* ntot, const int* start, int* fill, int* perm,
                    cudaStream_t s)
{
    if (ncap <= 0) return;
    k_scatter<<<(ncap + 255) / 256, 256, 0, s>>>(cell_of, ntot, start, fill, perm);
}

// Rank sort of each cell's entries by (z, index) (a warp per cell, persistent
// over the actual cells): entry v goes to slot start + #{u in cell : (z_u, u) <
// (z_v, v)}, z the coordinate wrapped in FP32.  Consecutive targets
// then lie close in z, which narrows the z-range of a real-space work item.
// Cells of more than kSortMax entries keep the (index) scatter order.
constexpr int kSortMax = 1024;

__global__ void k_sort_cells(const int* __restrict__ perm_in, int* __restrict__ perm_out,
                             const int* __restrict__ start, const int* __restrict__ cell_offsets,
                             const PbInst* __restrict__ inst, int ninst, const double* __restrict__ pos)
{
    const int ncell = cell_offsets[ninst];
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int cell = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; cell < ncell; cell += nwarps) {
        const int b = start[cell], e = start[cell + 1], n = e - b;
        if (n <= 1) {
            if (n == 1 && lane == 0) perm_out[b] = perm_in[b];
            continue;
        }
        const int q = find_instance(cell_offsets, ninst, cell);
        if (n > kSortMax) {
            for (int i = lane; i < n; i += 32) perm_out[b + i] = perm_in[b + i];
            continue;
        }
        const PbInst& I = inst[q];
        // FP32 key (the order only shapes the work items; FP64 would cost the GPU's slow FP64 pipe)
        const float Lz = (float)I.L[2], iLz = (float)I.iL[2];
        auto zkey = [&](int v) {
            float z = (float)pos[3 * (size_t)v + 2];
            z -= Lz * floorf(z * iLz);
            return (z == z) ? z : 0.f;
        };
        for (int ib = 0; ib < n; ib += 32) {
            const int i = ib + lane;
            const int v = i < n ? perm_in[b + i] : 0;
            const float z = i < n ? zkey(v) : 0.f;
            int rank = 0;
            for (int jb = 0; jb < n; jb += 32) {
                const int j = jb + lane;
                const int u = j < n ? perm_in[b + j] : 0;
                const float zu = j < n ? zkey(u) : 0.f;
                const int m = min(32, n - jb);
                for (int k = 0; k < m; k++) {
                    const int uk = __shfl_sync(kFull, u, k);
                    const float zk = __shfl_sync(kFull, zu, k);
                    rank += (zk < z) || (zk == z && uk < v);
                }
            }
            if (i < n) perm_out[b + rank] = v;
        }
    }
}

void launch_sort_cells(int* perm, int* perm_tmp, const int* start, int ncell_cap, const int* cell_offsets,
                       const PbInst* inst, int ninst, const double* pos, int nsm, cudaStream_t s)
{
    if (ncell_cap <= 0) return;
    long long blocks = ((long long)ncell_cap * 32 + 255) / 256;
    if (blocks > (long long)nsm * 16) blocks = (long long)nsm * 16;
    k_sort_cells<<<(int)blocks, 256, 0, s>>>(perm, perm_tmp, start, cell_offsets, inst, ninst, pos);
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
// or where 32 targets would span more than 8 cells.  Each row item becomes
// `G` = csplit work items, one per group of stencil columns, so that small
// instances still fill the GPU.  One thread per row start: a counting walk,
// then the emitting walk into its range.  A row gives at most
// targets/32 + cells items.
// Item = {instance, first target, local row, count | za << 8 | zb << 16 | group << 24}.
template <bool EMIT>
__device__ void walk_row(const int* __restrict__ start, int row0, int nz, int q, int rowl, int G, int4* items,
                         int k0, int cap, int& nitems)
{
    int k = 0, z = 0;
    int t = start[row0];
    const int end = start[row0 + nz];
    while (t < end) {
        while (start[row0 + z + 1] <= t) z++;  // za: the cell of target t
        const int za = z;
        const int lim = min(min(t + 32, end), start[row0 + min(za + 8, nz)]);
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
                const int G = max(1, I.csplit);
                int n = 0;
                walk_row<false>(st[w], 0, nz, rq, rl / nz, G, nullptr, 0, 0, n);
                if (n > 0) {
                    const int k0 = atomicAdd(nitems, n);
                    if (k0 + n > cap) atomicOr(status, kCapItems);  // items dropped: reported, not silent
                    walk_row<true>(st[w], 0, nz, rq, rl / nz, G, items, k0, cap, n);
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

}  // namespace pb

namespace pb {

__global__ void k_pack_targets(const double* __restrict__ x, const double* __restrict__ y,
                               const int* __restrict__ tgt_off, const int* __restrict__ src_off,
                               const int* __restrict__ y_off, int ninst, double* __restrict__ out)
{
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= tgt_off[ninst]) return;
    int q = find_instance(tgt_off, ninst, p);
    int local = p - tgt_off[q];
    const double* src = (y_off[q] >= 0) ? (y + 3 * (size_t)(y_off[q] + local)) : (x + 3 * (size_t)(src_off[q] + local));
    out[3 * (size_t)p] = src[0];
    out[3 * (size_t)p + 1] = src[1];
    out[3 * (size_t)p + 2] = src[2];
}

void launch_pack_targets(const double* x, const double* y, int ncap, const int* tgt_off, const int* src_off,
                         const int* y_off, int ninst, double* out, cudaStream_t s)
{
    if (ncap <= 0) return;
    k_pack_targets<<<(ncap + 255) / 256, 256, 0, s>>>(x, y, tgt_off, src_off, y_off, ninst, out);
}

}  // namespace pb
