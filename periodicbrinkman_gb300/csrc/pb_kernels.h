// Launch wrappers for the CUDA kernels of the evaluator (host-callable).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "pb_types.h"

namespace pb {

// ---- binning and sorting (pb_sort.cu) ----
// Every particle kernel is launched for a capacity `ncap` and reads the actual
// count from device memory (offsets[ninst]), so one captured graph serves any
// set of instances that fits the capacity.
// Sorted particle records again from the permutation of the last cell-list
// build (new forces at the same positions).  Mixed: pos_hi (x,y,z, w =
// instance bits), pos_lo, frc.  Non-finite coordinates and forces are replaced
// by 0 and set bad[instance] = 1 (bad may be null).
void launch_prepare_mixed(const double* pos, const double* frc, const int* perm, int ncap, const int* offsets,
                          const PbInst* inst, int ninst, float4* pos_hi, float4* pos_lo, float4* frc_out, int* bad,
                          cudaStream_t s);
void launch_prepare_fp64(const double* pos, const double* frc, const int* perm, int ncap, const int* offsets,
                         const PbInst* inst, int ninst, Dbl4* pos_out, Dbl4* frc_out, int* bad, cudaStream_t s);
// Cell lists of the sources and, when they have their own, of the targets, in
// four launches shared by both sets: binning (cell, arrival slot and z key of
// every particle), one decoupled look-back scan per set, the scatter, and a
// thread per particle ranking it in its cell by (wrapped z as FP32, index)
// and writing its sorted record.  Instance q's targets are read from y when
// y_off[q] >= 0, else they are its sources.  The zero region (counts, scan
// flags, tickets; cell_list_zero_bytes) must be zeroed before every build.
struct CellListArgs {
    const double *x, *f, *y;
    const int *src_off, *tgt_off, *y_off, *cell_off;
    const PbInst* inst;
    int ninst;
    int ncap_s, ncap_t;   // launch capacities
    int two;              // the targets have their own cell list (else they are the sources)
    int ncell_cap;
    int cstride, ntiles;  // set by launch_cell_lists: count stride, scan tiles per set
    int4 *key_s, *key_t;  // per particle: {global cell, arrival slot in it, instance, z key bits}
    int* zero;            // zero region: counts [2][cstride], tickets, look-back flags
    int* start;           // cell starts [2][cstride] (targets at cstride)
    int2 *perm_tmp_s, *perm_tmp_t;  // per cell, in arrival order: {particle, z key bits}
    int *perm_s, *perm_t;           // sorted position -> particle
    void *spos_a, *spos_b, *sfrc, *tpos_a, *tpos_b;  // records (mixed: hi, lo, force; FP64: pos, force)
    int* bad;             // per instance, then the execution status word at [ninst]
};
int cell_list_stride(int ncell_cap);
size_t cell_list_zero_bytes(int ncell_cap);
void launch_cell_lists(const CellListArgs& a, bool mixed, int nsm, cudaStream_t s);
// Work items: up to 32 consecutive targets of one cell row spanning <= kItemCells cells,
// times csplit stencil column groups:
// int4 {inst, first target, local row, count | za << 8 | zb << 16 | group << 24}.
// Builds the items of all row-start cells (cell_offsets[ninst] = actual cells);
// *nitems = number of items.  Items beyond `cap` are not written: the
// real-space kernels clamp to cap and *status gets kCapItems, which the host
// turns into an error.
void launch_build_items(const int* start, int ncell_cap, const int* cell_offsets, const PbInst* inst, int ninst,
                        int4* items, int cap, int* nitems, int* status, int nsm, cudaStream_t s);

// ---- real space (pb_real.cu) ----
// Mixed precision: FP32 polynomial kernel, hi/lo displacements, Kahan sums.
// Both kernels zero u_real (3 doubles per target, ntgt_cap targets) and add
// each work item's part into it with FP64 atomics.
void launch_real_mixed(int npoly, const PbInst* inst, const PbTables* tab, const int4* items, const int* nitems_ptr,
                       int nitems_max, const float4* spos_hi, const float4* spos_lo, const float4* sfrc,
                       const int* src_start, const float4* tpos_hi, const float4* tpos_lo, int ntgt_cap,
                       double* u_real, int* counter, int nsm, cudaStream_t s);
// FP64: closed forms of the reference with the FP64 series below r_tiny.
void launch_real_fp64(const PbInst* inst, const PbTables* tab, const int4* items, const int* nitems_ptr,
                      int nitems_max, const Dbl4* spos, const Dbl4* sfrc, const int* src_start,
                      const Dbl4* tpos, int ntgt_cap, double* u, int* counter, int nsm, cudaStream_t s);

// ---- k space (pb_kspace.cu) ----
template <class T>
void launch_spread(const PbInst* inst, int ninst, const int* src_offsets, int ncap, const void* pos_a,
                   const void* pos_b, const void* frc, T* grid, cudaStream_t s);
template <class T>
void launch_gather(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const void* pos_a,
                   const void* pos_b, const T* grid, T* u_k, cudaStream_t s);
// Batched 3D R2C -> Green multiply -> C2R over `nvol` volumes of equal size
// (3 components per instance, instances contiguous).
template <class T>
void launch_kspace_fft(const PbInst* inst_dev, const int* bucket_inst, int ninst_bucket, long long base_off,
                       const int* M, T* grid, void* spec, const void* twiddles, cudaStream_t s);
// FP32 grids of one grid-size bucket, tile by tile (pb_spread.cu): `nb`
// instances bucket_inst[0..nb) of grid M, points from the source cell list
// (src_start, sorted records); every tile of a live instance is written
// whole, so the grids need no clearing.
void launch_spread_tiles(const PbInst* inst, const int* bucket_inst, int nb, const int* M, const int* src_start,
                         const float4* pos_a, const float4* pos_b, const float4* frc, float* grid, cudaStream_t s);
// Zeroes the grids (4 M^3 elements of esz bytes) of instances with sources or targets.
void launch_zero_grids(const PbInst* inst, int ninst, void* grid, int esz, cudaStream_t s);
size_t twiddle_bytes(const int* M, bool fp64);
void fill_twiddles(const int* M, bool fp64, void* host_buf);

// ---- final combine ----
void launch_combine_mixed(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const int* tperm,
                          const double* u_real, const float* u_k, int use_real, int use_k, const double* fsum,
                          const PbTables* tab, const double* frc, const int* src_offsets, double* U, cudaStream_t s);
void launch_combine_fp64(const PbInst* inst, int ninst, const int* tgt_offsets, int ncap, const int* tperm,
                         const double* u_real, const double* u_k, int use_real, int use_k, const double* fsum,
                         const PbTables* tab, const double* frc, const int* src_offsets, double* U, cudaStream_t s);
// Per-instance force sums (for the optional k = 0 mode): out[3*q + c] = sum f.
void launch_force_sums(const PbInst* inst, const double* frc, const int* offsets, int ninst, double* out,
                       cudaStream_t s);

// ---- dense mobility matrix (pb_dense.cu) ----
int launch_dense_matrix(double* dA, const double* dx, int m, const double* dx0, int n, double a, double d, double e,
                        const int* Mx, const int* Nx, const double* L, int tau_scaled, cudaStream_t s);

}  // namespace pb
