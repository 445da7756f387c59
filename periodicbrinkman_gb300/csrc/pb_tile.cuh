// Device helpers of the tiled kernels (pb_spread.cu): a block-wide scan for
// 256 threads, the range of real-space cells whose points reach a grid tile,
// and a positive modulo.
#pragma once
#include "pb_device.cuh"

namespace pb {

// Block-wide exclusive prefix sum of v over 256 threads; the total in *total.
// wsum holds 9 ints of shared memory (reused between calls).
__device__ __forceinline__ int block_scan256(int v, int* wsum, int* total)
{
    constexpr int kThreads = 256;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();  // wsum is reused between calls
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int base = 0, tot = 0;
#pragma unroll
    for (int k = 0; k < kThreads / 32; k++) {
        const int s = wsum[k];
        base += k < w ? s : 0;
        tot += s;
    }
    *total = tot;
    return base + x - v;
}

// Cells of one axis that meet the physical range [lo h, hi h) (grid units
// lo, hi; h the grid spacing), as a first cell (any integer, taken mod nc)
// and a count (nc: all of them).
__device__ __forceinline__ void cell_span(const PbInst& I, int a, int lo, int hi, int& first, int& count)
{
    const int cl = (int)floor((double)lo * I.gh[a] * I.ih[a] - 1e-9);
    const int ch = (int)floor((double)hi * I.gh[a] * I.ih[a] + 1e-9);
    count = ch - cl + 1;
    if (count >= I.nc[a]) {
        first = 0;
        count = I.nc[a];
    } else {
        first = cl;
    }
}

// Cells of one axis whose points can reach grid indices [t0, t0 + T) through a
// window of P points: physical range [(t0 - P/2 - 1) h, (t0 + T + P/2) h) (one
// grid cell of margin each side for the FP32 cell of a point).
__device__ __forceinline__ void cell_range(const PbInst& I, int a, int t0, int T, int& first, int& count)
{
    cell_span(I, a, t0 - I.Pa[a] / 2 - 1, t0 + T + I.Pa[a] / 2, first, count);
}

__device__ __forceinline__ int pmod(int v, int n)
{
    const int r = v % n;
    return r < 0 ? r + n : r;
}

}  // namespace pb
