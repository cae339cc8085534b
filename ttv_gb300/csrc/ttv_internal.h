// Internal interface between the C-ABI translation units (not installed).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>

#include <string>

#include "../../include/tlibg.h"
#include "ttv_kernels.cuh"

namespace tlibg {

// NVTX range over one C-ABI call (header-only NVTX: a no-op unless a
// profiler such as Nsight Systems attaches).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct CanonView {
    uint64_t P = 1, nq = 1, S = 1;
    int ref_case = 0;
};

// Validate a low-level call exactly like tlibg_ttv_* and reduce it to the
// canonical (S, nq, P) view; sets the thread's last error on failure.
int internal_analyse(size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
                     const size_t* pia, const void* b, const size_t* nb, const void* c,
                     const size_t* nc, const size_t* wc, const size_t* pic, CanonView* out);
// The single-call planner (heuristic).
int internal_plan(int dtype, const CanonView& cn, const void* a, const void* b,
                  const tlibg_options* opt, int sms, Plan* out);
// Streaming multiprocessors of the current device (0 without a device).
int internal_sms();
// Refuse pageable host pointers among a, b, c (sets the last error).
int internal_check_device_pointers(const void* a, const void* b, const void* c);
int internal_fail(int code, const std::string& msg);
int internal_ok();
int internal_cuda_fail(cudaError_t e, const char* where);
// cudaMalloc, counted by tlibg_device_alloc_count (every device allocation of
// the library goes through it).
cudaError_t internal_malloc(void** p, size_t bytes);
// The calling stream's cached device scratch (grow-only, per device and
// stream), at least `bytes` long; 256-byte aligned.
int internal_scratch(cudaStream_t stream, size_t bytes, void** out);
void internal_count_launches(uint64_t n);

}  // namespace tlibg
