// Kernel launch interface shared by the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tlibg {

enum DType { F32 = 0, F64 = 1, BF16A = 2 };
enum Kind { KIND_ROW = 0, KIND_COL = 1 };

constexpr int BLOCK = 256;            // threads per CTA for every TTV kernel
constexpr int BSTAGE_BYTES = 16384;   // bytes of b staged per CTA by the column kernel

// One planned launch of a canonical problem C[s, j] = sum_i A[s, i, j] b[i],
// A dense (S, nq, P) row-major, C dense (S, P).
struct Plan {
    int dtype = F32;
    int kind = KIND_COL;
    int group = 1;        // ROW: lanes per output row; COL: warps along the contracted mode
    int vec = 1;          // elements per vector load
    int split = 1;        // segments of the contracted mode
    int kahan = 1;        // compensated fp32 accumulation
    uint64_t P = 1, nq = 1, S = 1;
    uint64_t seg_len = 1;
    uint64_t items = 0;          // work items (ROW: rows x segments; COL: tiles x segments)
    uint64_t items_per_cta = 0;  // COL: contiguous block of items per CTA
    int grid = 1;
    size_t smem = 0;
    bool f64_combine = false;    // combine split partials in fp64 (fp32 storage, nq > 2^20)
};

struct KArgs {
    const void* a;
    const void* b;
    void* out;        // C (split == 1) or nothing
    void* partial;    // split partials (Pair<T>[split][S*P]) when split > 1
    uint64_t S, nq, P;
    uint64_t seg_len;
    uint64_t items, items_per_cta, ntiles;
    uint32_t nseg;
    uint32_t group;
};

// Bytes of partial storage a plan needs (0 when split == 1).
size_t partial_bytes(const Plan& p);

// Enqueue the plan's kernels (main kernel and, when split > 1, the combine).
// `partial` must hold partial_bytes(plan) bytes.  Returns cudaSuccess or the
// launch error.  Adds the number of launched kernels to *launches.
cudaError_t launch_plan(const Plan& plan, const void* a, const void* b, void* c, void* partial,
                        cudaStream_t stream, uint64_t* launches);

// Dynamic shared memory and the occupancy-derived CTAs per SM of a plan's
// main kernel (cached per instantiation).
size_t plan_smem_bytes(const Plan& p);
int plan_ctas_per_sm(const Plan& p);

unsigned int read_and_clear_device_error();

}  // namespace tlibg
