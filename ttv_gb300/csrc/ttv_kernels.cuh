// Kernel launch interface shared by the C-ABI layer and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tlibg {

enum DType { F32 = 0, F64 = 1, BF16A = 2 };
enum Kind {
    KIND_ROW = 0, KIND_COL = 1, KIND_STREAM = 2, KIND_COL_REALIGN = 3, KIND_COL_THIN = 4, KIND_ROW_TILE = 5,
    KIND_COL_BULK = 6, KIND_ROW_PANEL = 7, KIND_ROW_SHIFT = 8
};

constexpr int BLOCK = 256;            // threads per CTA for every TTV kernel
// SM count assumed by tlibg_plan when no device is present (a GB300: 2 dies x
// 76 SMs); every launch plans with the current device's own count.
constexpr int PLAN_SMS_WITHOUT_DEVICE = 152;
constexpr int BSTAGE_BYTES = 16384;   // bytes of b staged per CTA by the column kernel
constexpr int STREAM_STAGE_BYTES = 16384;   // streamed kernel: bytes of A per shared-memory stage
constexpr int STREAM_CONSUMERS = 256;       // streamed kernel: consumer threads per CTA
// Longest contraction of the short-contraction column kernel.
constexpr int CS_MAXQ = 4;
// TMA-staged column kernel: bytes of A per row of a tile (4 KB), a stage's row
// slot (plus the cover's misalignment), rows per stage, stages, threads
constexpr int CB_ROW_BYTES = 4096;
constexpr int CB_ROWB = CB_ROW_BYTES + 16;
constexpr int CB_RB = 8;
constexpr int CB_NS = 3;
constexpr int CB_CONSUMERS = BLOCK;                // consumer threads (512 measured slower)
constexpr int CB_THREADS = CB_CONSUMERS + 32;      // and a producer warp
// row-tile kernel: warps per CTA, shared-memory stages per warp, longest row
constexpr int ROWT_WARPS = 4;
constexpr int ROWT_THREADS = ROWT_WARPS * 32;
constexpr int ROWT_NS = 2;
constexpr int ROWT_MAX_NQ = 64;
// Bytes of one row-tile stage: 32 R rows of n_q elements of A plus up to 15
// bytes of misalignment, rounded to 16.
__host__ __device__ inline size_t rowt_slot_bytes(uint64_t nq, size_t ea, int R)
{
    return (size_t)((32 * (uint64_t)R * nq * ea + 16 + 15) & ~uint64_t(15));
}
// Row-panel kernel: vectors of b each thread holds in registers; a segment is
// RP_K * BLOCK vectors.
constexpr int RP_K = 4;
inline uint64_t row_panel_seg(int dtype) { return (uint64_t)RP_K * BLOCK * (dtype == F64 ? 2 : (dtype == BF16A ? 8 : 4)); }
// Outputs per tile of the TMA-staged column kernel (4 KB of A per row).
inline uint64_t col_bulk_tile(int dtype) { return (uint64_t)CB_ROW_BYTES / (dtype == F64 ? 8 : (dtype == BF16A ? 2 : 4)); }
// Rows per lane of a row tile: enough that a tile holds about 4 KB of A.
inline int rowt_rows_per_lane(uint64_t nq, size_t ea)
{
    const uint64_t b = 32 * nq * ea;
    return b >= 4096 ? 1 : (2 * b >= 4096 ? 2 : 4);
}

// One planned launch of a canonical problem C[s, j] = sum_i A[s, i, j] b[i],
// A dense (S, nq, P) row-major, C dense (S, P).
struct Plan {
    int dtype = F32;
    int kind = KIND_COL;
    int group = 1;        // ROW: lanes per output row; COL / COL_REALIGN: warps along the contracted mode
    int vec = 1;          // elements per vector load (COL_REALIGN: 16 bytes, realigned by shuffles)
    int split = 1;        // segments of the contracted mode
    int kahan = 1;        // compensated fp32 accumulation
    int rows_m = 0;       // ROW: 1 or 2 = short-row kernel (at most rows_m vectors per lane of a row);
                          // COL: 1 = short-contraction kernel (n_q <= CS_MAXQ, two tiles per thread);
                          // ROW_TILE: rows per lane (1, 2 or 4); ROW_PANEL: rows in flight (1 or 2)
    int mo = 1;           // COL with scalar loads: outputs per thread, 32 apart (strided kernel when > 1)
    uint64_t P = 1, nq = 1, S = 1;
    uint64_t seg_len = 1;
    uint64_t items = 0;          // work items (ROW: rows x segments; COL: tiles x segments;
                                 //   ROW_PANEL: segments x row blocks)
    uint64_t items_per_cta = 0;  // COL: contiguous block of items per CTA; ROW_PANEL: rows per row block
    int grid = 1;
    int sms = 0;                 // streaming multiprocessors of the device planned for
    size_t smem = 0;
    bool f64_combine = false;    // combine split partials in fp64 (fp32 storage, nq > 2^20)
    // streamed kernel (kind == KIND_STREAM): A as rows of L elements, R rows per chunk
    int stream_col = 0;          // 0: row form (P == 1), 1: column form
    uint64_t L = 0, R = 0, units = 0, units_per_cta = 0;
    int RG = 1, J = 1;
};

// Row-shift kernel (rows that are not whole 16-byte vectors): V shifted copies
// of b, each W = n_q + V rounded up to V elements, plus their double-float
// splits for fp64 with the mix; at most RS_SMEM_MAX bytes.
constexpr size_t RS_SMEM_MAX = 48 * 1024;
__host__ __device__ inline uint64_t rs_width(uint64_t nq, int V) { return (nq + V + V - 1) / V * V; }
__host__ __device__ inline size_t rs_smem_bytes(uint64_t nq, size_t es, bool split)
{
    const int V = (int)(16 / es);
    const uint64_t W = rs_width(nq, V);
    return (size_t)V * W * es + (split ? (size_t)V * W * 8 : 0);
}

// Whether the streamed kernel can take a problem (whole rows fit a stage).
bool stream_eligible(int dtype, uint64_t P, uint64_t nq);

// --------------------------------------------------------------------------
// division by a divisor fixed for a launch (output -> slice, item -> segment)
// --------------------------------------------------------------------------
// When every dividend and the divisor fit 32 bits, n / d is one multiply-high,
// a subtract, an add and two shifts: the round-up method of Granlund and
// Montgomery ("Division by invariant integers using multiplication", PLDI
// 1994, section 4) with l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1,
// t = hi32(m n), n / d = (t + ((n - t) >> min(l, 1))) >> max(l - 1, 0).
// Otherwise the plain 64-bit division.  Built on the host per launch (and on
// the device per problem by the batched executor's planning kernel).
struct IdxDiv {
    uint64_t d;
    uint32_t m;
    uint8_t s1, s2, fast;
};

__host__ __device__ inline IdxDiv make_idx_div(uint64_t d, uint64_t max_dividend)
{
    IdxDiv v{d == 0 ? 1 : d, 0, 0, 0, 0};
    if (v.d < (uint64_t(1) << 32) && max_dividend < (uint64_t(1) << 32)) {
        uint32_t l = 0;
        while ((uint64_t(1) << l) < v.d) ++l;
        v.m = (uint32_t)(((uint64_t(1) << 32) * ((uint64_t(1) << l) - v.d)) / v.d + 1);
        v.s1 = (uint8_t)(l < 1 ? l : 1);
        v.s2 = (uint8_t)(l > 0 ? l - 1 : 0);
        v.fast = 1;
    }
    return v;
}

// (Host-callable too, so the CPU tests run this very code.)
__host__ __device__ __forceinline__ uint64_t idx_div(uint64_t n, const IdxDiv& v)
{
    if (v.fast) {
        const uint32_t x = (uint32_t)n;
#ifdef __CUDA_ARCH__
        const uint32_t t = __umulhi(v.m, x);
#else
        const uint32_t t = (uint32_t)(((uint64_t)v.m * x) >> 32);
#endif
        return (t + ((x - t) >> v.s1)) >> v.s2;
    }
    return n / v.d;
}

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
    IdxDiv pdiv;      // outputs -> slice (division by P)
    IdxDiv tdiv;      // items -> segment (division by ntiles)
};

// Bytes of partial storage a plan needs (0 when split == 1).
size_t partial_bytes(const Plan& p);

// Enqueue the plan's kernels (main kernel and, when split > 1, the combine).
// `partial` must hold partial_bytes(plan) bytes.  Returns cudaSuccess or the
// launch error.  Adds the number of launched kernels to *launches.  The
// combine is launched as a programmatic dependent of the main kernel; the
// main kernel too when `dependent` is set (its predecessor in the stream is
// an engine kernel of the same call).
cudaError_t launch_plan(const Plan& plan, const void* a, const void* b, void* c, void* partial,
                        cudaStream_t stream, uint64_t* launches, bool dependent = false);

// Second phase of a split plan: C[o] = sum over segments of the partials.
cudaError_t launch_combine(const Plan& plan, void* partial, void* c, cudaStream_t stream, uint64_t* launches);

// Dynamic shared memory and the occupancy-derived CTAs per SM of a plan's
// main kernel (cached per instantiation).
size_t plan_smem_bytes(const Plan& p);
int plan_ctas_per_sm(const Plan& p);

unsigned int read_and_clear_device_error();

// Self-test kernel: one bounded mbarrier wait that nothing completes.
cudaError_t launch_wait_probe(cudaStream_t stream, uint32_t limit);

}  // namespace tlibg
