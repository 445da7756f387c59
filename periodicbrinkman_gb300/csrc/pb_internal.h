// Library-internal entry points shared by the C ABI files (not exported in
// include/pbrinkman.h).
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "pb_types.h"
#include "pbrinkman.h"

namespace pb {

// An NVTX range over a scope of host code (API calls, server steps, the
// launch of each stage): visible in Nsight Systems timelines, free otherwise.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Sets the calling thread's pb_last_error() message; returns `code`.
int api_error(int code, const char* msg);
// Descriptor of one k-space-only instance with all offsets 0.
int kspace_instance(const pb_solve_params& p, PbInst* inst);
// Resolved parameters of one instance without its tables (npoly = 0).
int resolve_info(const pb_solve_params& p, pb_instance_info* info);
// Resolved parameters and real-space tables of one instance, built as a plan
// (or slot) whose far polynomial holds `npoly_cap` terms builds them.
int prepare_instance(const pb_solve_params& p, int npoly_cap, PbTables* tab, pb_instance_info* info);
// pb_plan_bind with tables from prepare_instance (tabs[q] belongs to p[q]).
int plan_bind_prepared(pb_plan P, const pb_solve_params* p, const PbTables* tabs, int count);
// Executes a bound plan with per-instance host buffers: instance q reads
// xs[q], fs[q] (and ys[q] when it has its own targets) and writes Us[q].
// Page-locked buffers are copied asynchronously; non-finite inputs are
// reported by plan_bad_flags.
int plan_execute_parts(pb_plan P, const double* const* xs, const double* const* fs, const double* const* ys,
                       double* const* Us, cudaStream_t stream);

// After an execution by plan_execute_parts has completed: flags[q] != 0 when
// instance q had a non-finite input (those inputs were computed as 0).
const int* plan_bad_flags(pb_plan P);
// After such an execution: its capacity status bits (kCapItems, ...).
int plan_exec_status(pb_plan P);

}  // namespace pb
