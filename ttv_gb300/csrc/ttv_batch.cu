// Batched TTVs in one persistent launch driven by a device-side work queue.
//
// A batch of independent fp32 problems (any order, extents, q and layout) is
// turned into device descriptors once (tlibg_batch_create).  Every launch is
// one short sequence, captured in a CUDA graph and replayed:
//
//   batch_select  (learned mode, once at creation: the scores depend only on
//                 the descriptors) the cost-model MLP scores every kernel
//                 variant of every problem and keeps the cheapest
//   batch_plan    one CTA: decodes each problem's variant into work units,
//                 prefix-sums units and split-partial offsets, fills the
//                 unit -> problem map and resets the queue
//   batch_exec    persistent CTAs (SMs x occupancy) pop units from an atomic
//                 counter; a unit is a block of rows (row form) or a tile of
//                 the prefix over one segment of q (column form); the CTA
//                 that completes a split problem's last unit combines its
//                 partials in fixed segment order
//   batch_rowtile persistent warps for the problems staged in shared memory
//                 (variant 8: short q-fastest rows): each warp pops units of
//                 tiles of 32 R rows, moves every tile into its own two-stage
//                 ring with one TMA bulk copy and walks one row per lane from
//                 shared memory (coalesced HBM reads, conflict-free walks)
//
// Variants (9): index v = 2*g + s for v < 8.  Row form: lanes per row
// G = 1 << g; column form: warps along q WI = 1 << g.  s = 1 splits q into up
// to 4 segments (two-phase, deterministic).  v = 8: row form with n_q <= 64,
// rows staged through shared memory (batch_rowtile); not valid for columns.
#include "ttv_device.cuh"
#include "ttv_internal.h"
#include "ttv_rowwalk.cuh"
#include "ttv_mlp.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

namespace tlibg {

static __device__ unsigned int g_batch_error = 0u;

struct BPair {
    float s, c;
};

struct BProb {
    const float* a;
    const float* b;
    float* c;
    uint64_t P, nq, S;
    uint64_t seg_len;
    uint64_t unit_begin;   // first unit of the problem in its executor's unit space
    uint64_t part_off;     // in BPair elements
    uint64_t tiles;        // column units: tiles per segment
    uint64_t tpu;          // column units: tiles per unit
    uint64_t upseg;        // column units: units per segment
    IdxDiv pdiv;           // column units: output -> slice (division by P)
    IdxDiv tdiv;           // column units: unit -> segment (division by the units per segment)
    IdxDiv sdiv;           // row units: item -> row (division by the segment count)
    float feat[NFEAT];
    int kind;
    int vec;
    int variant;
    int group;
    uint32_t nseg;
    uint32_t units;
    uint32_t valid_mask;
    int heuristic;               // the fixed rule's variant (kept unless the model beats it by the margin)
    int staged;                  // this launch runs the problem in batch_rowtile (variant 8)
    int cls;                     // executor class of this launch (CLS_*)
    unsigned int done;
    unsigned long long cycles;   // SM clock cycles spent on this problem's units (recording launches)
};

// Executor classes, one persistent kernel each (launched in turn):
//   CLS_GENERIC  row units (lane groups) and column units with 16-byte loads
//   CLS_COL1     column units with scalar or 8-byte loads (prefixes that are
//                odd, or even but not a multiple of 4): two vectors per thread
//                32 vectors apart, running row pointers, more loads in flight
//   CLS_STAGED   staged short rows (variant 8)
constexpr int CLS_GENERIC = 0, CLS_COL1 = 1, CLS_STAGED = 2, NCLS = 3;

struct BCtl {
    unsigned long long head[NCLS];    // each class's queue: next unit to hand out
    unsigned long long total[NCLS];   // each class's units
    int record;                       // nonzero: accumulate per-problem unit cycles
};

// Staged row units (variant 8, batch_rowtile): tiles of 32 R rows of at most
// BRT_TILE_BYTES, BRT_TPU tiles per work unit, one two-stage ring per warp.
constexpr int VARIANT_STAGED = 8;
constexpr int BRT_WARPS = 4;
constexpr int BRT_THREADS = BRT_WARPS * 32;
constexpr int BRT_NS = 2;
constexpr int BRT_MAX_NQ = 64;
constexpr int BRT_TILE_BYTES = 8192;
constexpr int BRT_SLOT = BRT_TILE_BYTES + 32;   // + the run's misalignment (< 16 bytes)
constexpr int BRT_TPU = 8;
constexpr size_t BRT_WARP_BYTES = (size_t)BRT_NS * (BRT_MAX_NQ * 4 + BRT_SLOT);
constexpr size_t BRT_SMEM = 128 + BRT_WARPS * BRT_WARP_BYTES;
// rows per lane of a tile: 32 R rows of n_q floats fill at most BRT_TILE_BYTES
__host__ __device__ inline uint32_t brt_rows_per_lane(uint64_t nq) { return nq <= 16 ? 4u : (nq <= 32 ? 2u : 1u); }
__host__ __device__ inline uint64_t brt_units(uint64_t nq, uint64_t S)
{
    const uint64_t tiles = (S + 32 * brt_rows_per_lane(nq) - 1) / (32 * brt_rows_per_lane(nq));
    return (tiles + BRT_TPU - 1) / BRT_TPU;
}

constexpr int BMAX_F32 = BSTAGE_BYTES / 4;

// Lanes per row of the row-form variants: G = TLIBG_BATCH_ROW_G0 << g, g = 0..3.
// Measured on GB300 (22,000 tuned shapes in mixed batches): one lane per row is
// the best single variant for the batch's rows of 8-512 elements (regret 4.5 %
// against 13.5 % for four lanes), and with G in {1, 2, 4, 8} the learned
// selection gains 8 % over a fixed four lanes in the 4096-problem launch.
#ifndef TLIBG_BATCH_ROW_G0
#define TLIBG_BATCH_ROW_G0 1
#endif

__host__ __device__ inline void decode_variant(int kind, int v, uint64_t nq, int* group, uint32_t* nseg)
{
    if (v == VARIANT_STAGED) {   // one lane per row from shared memory, no split
        *group = 1;
        *nseg = 1;
        return;
    }
    const int gi = (v >> 1) & 3, si = v & 1;
    *group = kind == KIND_ROW ? (TLIBG_BATCH_ROW_G0 << gi) : (1 << gi);
    uint64_t ns = 1;
    if (si) ns = nq >= 64 ? 4 : (nq >= 16 ? 2 : 1);
    const uint64_t min_seg = kind == KIND_COL ? (nq + BMAX_F32 - 1) / BMAX_F32 : 1;
    if (ns < min_seg) ns = min_seg;
    if (ns > nq) ns = nq;
    *nseg = (uint32_t)ns;
}

// Bytes of A a work unit covers: enough that the per-unit latency (claiming it,
// its problem's descriptor, the first loads' round trip) is small next to the
// unit's streaming time, few enough that the launch still ends level.
#ifndef TLIBG_BATCH_UNIT_BYTES
#define TLIBG_BATCH_UNIT_BYTES 131072
#endif

// Row form: rounds of one row segment per lane group that make up a work unit.
__host__ __device__ inline uint64_t rows_per_group(uint64_t seg_len, int group)
{
    const uint64_t gpc = BLOCK / group;
    const uint64_t per_round = gpc * seg_len * 4;
    uint64_t r = (TLIBG_BATCH_UNIT_BYTES + per_round - 1) / per_round;
    return r < 1 ? 1 : (r > 256 ? 256 : r);
}

// Column form: vectors per thread (two, 32 vectors apart, for scalar and
// 8-byte loads) and outputs per tile (the CTA's warp rows of 32 lanes).
constexpr int COL1_MO = 2;
__host__ __device__ inline uint64_t col_tile_outputs(int group, int vec)
{
    return (uint64_t)((BLOCK / 32) / group) * 32 * vec * (vec <= 2 ? COL1_MO : 1);
}

// Column form: a unit is `tpu` consecutive tiles of one segment.
__host__ __device__ inline uint64_t tiles_per_unit(uint64_t TO, uint64_t seg_len, uint64_t tiles)
{
    uint64_t t = TLIBG_BATCH_UNIT_BYTES / (TO * seg_len * 4);
    if (t < 1) t = 1;
    return t > tiles ? tiles : t;
}

__host__ __device__ inline uint64_t unit_count(int kind, int group, int vec, uint64_t P, uint64_t nq,
                                               uint64_t S, uint32_t nseg, uint64_t* seg_len)
{
    uint64_t sl = (nq + nseg - 1) / nseg;
    if (kind == KIND_ROW) sl = (sl + vec - 1) / vec * vec;
    *seg_len = sl;
    const uint64_t ns = (nq + sl - 1) / sl;
    if (kind == KIND_ROW) {
        const uint64_t per_unit = (BLOCK / group) * rows_per_group(sl, group);
        return (S * ns + per_unit - 1) / per_unit;
    }
    const uint64_t TO = col_tile_outputs(group, vec);
    const uint64_t tiles = (S * P + TO - 1) / TO;
    const uint64_t tpu = tiles_per_unit(TO, sl, tiles);
    return (tiles + tpu - 1) / tpu * ns;
}

// --------------------------------------------------------------------------
// selection: MLP score per (problem, variant), keep the argmin
// --------------------------------------------------------------------------
// One thread per (problem, variant slot); SELECT_LANES slots per problem (a
// power of two >= NVARIANT, the unused ones score +inf).
constexpr int SELECT_LANES = 16;
static_assert(NVARIANT <= SELECT_LANES, "variant slots per problem");

__global__ void __launch_bounds__(256) batch_select(BProb* __restrict__ pr, int n, const float* __restrict__ w,
                                                    float log2_count, float log2_keep)
{
    __shared__ float sw[MLP_PARAMS];
    for (int p = threadIdx.x; p < MLP_PARAMS; p += blockDim.x) sw[p] = w[p];
    __syncthreads();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int pi = t / SELECT_LANES, v = t % SELECT_LANES;
    float score = INFINITY;
    if (pi < n && v < NVARIANT && ((pr[pi].valid_mask >> v) & 1u)) {
        float x[MLP_IN];
#pragma unroll
        for (int i = 0; i < NFEAT; ++i) x[i] = pr[pi].feat[i];
#pragma unroll
        for (int i = 0; i < NVARIANT; ++i) x[NFEAT + i] = (i == v) ? 1.f : 0.f;
        score = mlp_forward<false>(sw, x, nullptr, nullptr, nullptr);
    }
    int best = v;
    const int h = pi < n ? pr[pi].heuristic : 0;
    // the fixed rule's predicted cost, broadcast within the problem's lanes
    const float h_score = __shfl_sync(0xffffffffu, score, (threadIdx.x & ~(unsigned)(SELECT_LANES - 1)) + (unsigned)h);
    // argmin over the problem's lanes (ties: lowest variant)
#pragma unroll
    for (int off = SELECT_LANES / 2; off > 0; off >>= 1) {
        const float os = __shfl_xor_sync(0xffffffffu, score, off);
        const int ob = __shfl_xor_sync(0xffffffffu, best, off);
        if (os < score || (os == score && ob < best)) {
            score = os;
            best = ob;
        }
    }
    // deviate from the fixed rule only for a predicted gain beyond the margin
    if (pi < n && v == 0) pr[pi].variant = (isinf(score) || !(score < h_score + log2_keep)) ? h : best;
    (void)log2_count;
}

__global__ void batch_set_variant(BProb* __restrict__ pr, int n, int v)
{
    // a variant a problem cannot run (the staged rows of a column problem) keeps its fixed rule
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pr[i].variant = ((pr[i].valid_mask >> v) & 1u) ? v : pr[i].heuristic;
}

// --------------------------------------------------------------------------
// plan: units, prefix sums, unit -> problem map, queue reset (one CTA)
// --------------------------------------------------------------------------
constexpr int PLAN_SUMS = 4;   // units of the three executor classes, split partials

__global__ void __launch_bounds__(1024) batch_plan(BProb* __restrict__ pr, int n, BCtl* ctl)
{
    __shared__ unsigned long long s_sum[PLAN_SUMS][32];
    __shared__ unsigned long long carry[PLAN_SUMS];
    if (threadIdx.x < PLAN_SUMS) carry[threadIdx.x] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + threadIdx.x;
        unsigned long long x[PLAN_SUMS] = {0, 0, 0, 0};
        if (i < n) {
            BProb& P = pr[i];
            if (!((P.valid_mask >> P.variant) & 1u)) P.variant = P.heuristic;   // not runnable: the fixed rule
            P.staged = P.variant == VARIANT_STAGED ? 1 : 0;
            int group;
            uint32_t nseg;
            decode_variant(P.kind, P.variant, P.nq, &group, &nseg);
            uint64_t seg_len;
            const uint64_t u = unit_count(P.kind, group, P.vec, P.P, P.nq, P.S, nseg, &seg_len);
            nseg = (uint32_t)((P.nq + seg_len - 1) / seg_len);
            P.group = group;
            P.nseg = nseg;
            P.seg_len = seg_len;
            P.done = 0u;
            P.cycles = 0ull;
            const uint64_t outputs = P.S * P.P;
            if (P.kind == KIND_COL) {
                const uint64_t TO = col_tile_outputs(group, P.vec);
                P.tiles = (outputs + TO - 1) / TO;
                P.tpu = tiles_per_unit(TO, seg_len, P.tiles);
                P.upseg = (P.tiles + P.tpu - 1) / P.tpu;
                P.pdiv = make_idx_div(P.P, outputs);
                P.tdiv = make_idx_div(P.upseg, P.upseg * nseg);
            } else {
                P.tiles = 0;
                P.sdiv = make_idx_div(nseg, P.S * nseg);
            }
            P.cls = P.staged ? CLS_STAGED : (P.kind == KIND_COL && P.vec <= 2 ? CLS_COL1 : CLS_GENERIC);
            if (P.staged) {
                P.units = (uint32_t)brt_units(P.nq, P.S);
            } else {
                P.units = (uint32_t)u;
                x[3] = nseg > 1 ? (unsigned long long)nseg * outputs : 0ull;
            }
            x[P.cls] = P.units;
        }
        // inclusive warp scans, then across warps
        unsigned long long y[PLAN_SUMS];
#pragma unroll
        for (int c = 0; c < PLAN_SUMS; ++c) y[c] = x[c];
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
            for (int c = 0; c < PLAN_SUMS; ++c) {
                const unsigned long long o = __shfl_up_sync(0xffffffffu, y[c], off);
                if (lane >= off) y[c] += o;
            }
        }
        if (lane == 31) {
#pragma unroll
            for (int c = 0; c < PLAN_SUMS; ++c) s_sum[c][warp] = y[c];
        }
        __syncthreads();
        if (warp == 0) {
#pragma unroll
            for (int c = 0; c < PLAN_SUMS; ++c) {
                unsigned long long w = lane < (int)(blockDim.x >> 5) ? s_sum[c][lane] : 0ull;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const unsigned long long o = __shfl_up_sync(0xffffffffu, w, off);
                    if (lane >= off) w += o;
                }
                s_sum[c][lane] = w;   // inclusive prefix over warps
            }
        }
        __syncthreads();
        unsigned long long before[PLAN_SUMS];
#pragma unroll
        for (int c = 0; c < PLAN_SUMS; ++c) before[c] = carry[c] + (warp ? s_sum[c][warp - 1] : 0ull) + y[c] - x[c];
        if (i < n) {
            BProb& P = pr[i];
            P.part_off = before[3];
            P.unit_begin = before[P.cls];
        }
        __syncthreads();
        if (threadIdx.x < PLAN_SUMS) carry[threadIdx.x] += s_sum[threadIdx.x][(blockDim.x >> 5) - 1];
        __syncthreads();
    }
    if (threadIdx.x < NCLS) {
        ctl->total[threadIdx.x] = carry[threadIdx.x];
        ctl->head[threadIdx.x] = 0ull;
    }
}

// unit -> problem maps of the classes: one warp per problem, its lanes over its units
__global__ void batch_fill_maps(const BProb* __restrict__ pr, int n, uint32_t* __restrict__ map0,
                                uint32_t* __restrict__ map1, uint32_t* __restrict__ map2)
{
    const int i = (int)((blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5);
    const uint32_t lane = threadIdx.x & 31u;
    if (i >= n) return;
    const BProb& P = pr[i];
    uint32_t* map = P.cls == CLS_GENERIC ? map0 : (P.cls == CLS_COL1 ? map1 : map2);
    for (uint64_t k = lane; k < P.units; k += 32) map[P.unit_begin + k] = (uint32_t)i;
}

// Start of every launch of a planned batch: empty queues, completion counts and
// recorded cycles.
__global__ void batch_reset(BProb* __restrict__ pr, int n, BCtl* ctl)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        pr[i].done = 0u;
        pr[i].cycles = 0ull;
    }
    if (i < NCLS) ctl->head[i] = 0ull;
}

// --------------------------------------------------------------------------
// the persistent executor
// --------------------------------------------------------------------------
// Row units read A through L1 when a lane's loads are narrower than 16 bytes:
// the lanes of a group then cover a fraction of each 32-byte sector per load and
// the group's next loads ask for the rest.
#ifndef TLIBG_BATCH_ROW_L1
#define TLIBG_BATCH_ROW_L1 1
#endif
template <int V>
__device__ __forceinline__ void row_load(const float* p, float (&out)[V])
{
    if constexpr (TLIBG_BATCH_ROW_L1 && V < 4)
        load_a_l1<float, float, V>(p, out);
    else
        load_a<float, float, V>(p, out);
}

// V elements of b in one load (row problems: b is aligned to V floats and
// segments start on multiples of V).
#ifndef TLIBG_BATCH_BVEC
#define TLIBG_BATCH_BVEC 1
#endif
template <int V>
__device__ __forceinline__ void b_load(const float* p, float (&out)[V])
{
    if constexpr (!TLIBG_BATCH_BVEC) {
#pragma unroll
        for (int v = 0; v < V; ++v) out[v] = __ldg(p + v);
    } else if constexpr (V == 4) {
        const float4 t = __ldg(reinterpret_cast<const float4*>(p));
        out[0] = t.x;
        out[1] = t.y;
        out[2] = t.z;
        out[3] = t.w;
    } else if constexpr (V == 2) {
        const float2 t = __ldg(reinterpret_cast<const float2*>(p));
        out[0] = t.x;
        out[1] = t.y;
    } else {
        out[0] = __ldg(p);
    }
}

template <int V, bool KAHAN>
__device__ __forceinline__ void row_unit(const BProb& P, uint64_t lu, int G, BPair* __restrict__ part)
{
    const uint32_t lane = threadIdx.x & 31u, gl = lane & (uint32_t)(G - 1);
    const uint64_t gpc = BLOCK / G;
    const uint64_t items = P.S * P.nseg;
    const uint64_t R = rows_per_group(P.seg_len, G);
    constexpr int U = (int)sizeof(float) * V >= 16 ? 4 : 64 / ((int)sizeof(float) * V);
    constexpr int M = U / 2;
    if (P.nseg == 1 && P.nq % V == 0 && P.nq / V <= (uint64_t)G * M) {
        // short rows (at most U/2 vectors per lane): two rows of the group per
        // round with all their loads in flight together; b is the same for both
        const uint64_t nv = P.nq / V;
        for (uint64_t r = 0; r < R; r += 2) {
            const uint64_t item0 = (lu * R + r) * gpc + threadIdx.x / G;
            const uint64_t item1 = (lu * R + r + 1) * gpc + threadIdx.x / G;
            const bool valid0 = item0 < items;
            const bool valid1 = r + 1 < R && item1 < items;
            float a0[M][V], a1[M][V], bv[M][V];
#pragma unroll
            for (int t = 0; t < M; ++t) {
                const uint64_t kv = gl + (uint64_t)t * G;
                const bool in = kv < nv;
                if (in && valid0) row_load<V>(P.a + item0 * P.nq + kv * V, a0[t]);
                else {
#pragma unroll
                    for (int v = 0; v < V; ++v) a0[t][v] = 0.f;
                }
                if (in && valid1) row_load<V>(P.a + item1 * P.nq + kv * V, a1[t]);
                else {
#pragma unroll
                    for (int v = 0; v < V; ++v) a1[t][v] = 0.f;
                }
                if (in) {
                    b_load<V>(P.b + kv * V, bv[t]);
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v) bv[t][v] = 0.f;
                }
            }
            Acc<float, KAHAN> c0, c1;
            c0.init();
            c1.init();
#pragma unroll
            for (int t = 0; t < M; ++t)
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    c0.fma_add(a0[t][v], bv[t][v]);
                    c1.fma_add(a1[t][v], bv[t][v]);
                }
            for (int off = G >> 1; off > 0; off >>= 1) {
                const float s0 = __shfl_xor_sync(0xffffffffu, c0.s, off);
                const float k0 = __shfl_xor_sync(0xffffffffu, c0.c, off);
                const float s1 = __shfl_xor_sync(0xffffffffu, c1.s, off);
                const float k1 = __shfl_xor_sync(0xffffffffu, c1.c, off);
                c0.merge(s0, k0);
                c1.merge(s1, k1);
            }
            if (gl == 0) {
                if (valid0) P.c[item0] = c0.value();
                if (valid1) P.c[item1] = c1.value();
            }
        }
        return;
    }
    for (uint64_t r = 0; r < R; ++r) {
        const uint64_t item = (lu * R + r) * gpc + threadIdx.x / G;
        const bool valid = item < items;
        Acc<float, KAHAN> acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        uint64_t row = 0, seg = 0;
        if (valid) {
            row = P.nseg == 1 ? item : idx_div(item, P.sdiv);
            seg = item - row * P.nseg;
            const uint64_t ib = seg * P.seg_len;
            const uint64_t ie = min(P.nq, ib + P.seg_len);
            const float* ap = P.a + row * P.nq + ib;
            const float* bp = P.b + ib;
            const uint64_t n = ie - ib, nv = n / V;
            uint64_t kv = gl;
            for (; kv + (U - 1) * G < nv; kv += U * G) {
                float av[U][V], bv[U][V];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    row_load<V>(ap + (kv + u * G) * V, av[u]);
                    b_load<V>(bp + (kv + u * G) * V, bv[u]);
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v].fma_add(av[u][v], bv[u][v]);
            }
#pragma unroll 4
            for (; kv < nv; kv += G) {
                float av[V], bv[V];
                row_load<V>(ap + kv * V, av);
                b_load<V>(bp + kv * V, bv);
#pragma unroll
                for (int v = 0; v < V; ++v) acc[v].fma_add(av[v], bv[v]);
            }
            for (uint64_t e = nv * V + gl; e < n; e += G) acc[0].fma_add(__ldcs(ap + e), __ldg(bp + e));
        }
#pragma unroll
        for (int v = 1; v < V; ++v) acc[0].merge(acc[v].s, acc[v].c);
        for (int off = G >> 1; off > 0; off >>= 1) {
            const float os = __shfl_xor_sync(0xffffffffu, acc[0].s, off);
            const float oc = __shfl_xor_sync(0xffffffffu, acc[0].c, off);
            acc[0].merge(os, oc);
        }
        if (valid && gl == 0) {
            if (P.nseg == 1) {
                P.c[row] = acc[0].value();
            } else {
                BPair pr;
                pr.s = acc[0].s;
                pr.c = KAHAN ? acc[0].c : 0.f;
                part[P.part_off + seg * P.S + row] = pr;
            }
        }
    }
}

// column unit: `tpu` consecutive tiles of TO outputs over one segment; each
// warp row walks its 32 V outputs of every tile in turn (its loads of the next
// tile follow its last products of this one without a CTA barrier unless the
// warps along q reduce through shared memory)
template <int V, bool KAHAN>
__device__ __forceinline__ void col_unit(const BProb& P, uint64_t lu, int WI, float* red, BPair* __restrict__ part)
{
    const uint32_t WO = (BLOCK / 32) / WI;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t wi = warp % WI, wo = warp / WI;
    const uint64_t TO = (uint64_t)WO * 32u * V;
    const uint64_t outputs = P.S * P.P;
    const uint64_t seg = P.nseg == 1 ? 0 : idx_div(lu, P.tdiv);
    const uint64_t tile0 = (lu - seg * P.upseg) * P.tpu;
    const uint64_t tile1 = min(P.tiles, tile0 + P.tpu);
    const uint64_t ib = seg * P.seg_len;
    const uint64_t ie = min(P.nq, ib + P.seg_len);
    const uint64_t Pp = P.P, nq = P.nq;
    const float* __restrict__ A = P.a;
    // b is read through L1 (warp-uniform per row)
    const float* __restrict__ bs = P.b;
    constexpr int U = (int)sizeof(float) * V >= 16 ? 4 : 64 / ((int)sizeof(float) * V);

    for (uint64_t tile = tile0; tile < tile1; ++tile) {
        const uint64_t o0 = tile * TO + ((uint64_t)wo * 32u + lane) * V;
        const bool valid = o0 < outputs;
        Acc<float, KAHAN> acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        if (valid) {
            const uint64_t s = idx_div(o0, P.pdiv);
            const uint64_t j = o0 - s * Pp;
            const float* ap = A + (s * nq) * Pp + j;
            uint64_t i = ib + wi;
            for (; i + (U - 1) * WI < ie; i += U * WI) {
                float av[U][V];
#pragma unroll
                for (int u = 0; u < U; ++u) load_a<float, float, V>(ap + (i + u * WI) * Pp, av[u]);
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const float bb = __ldg(bs + i + u * WI);
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v].fma_add(av[u][v], bb);
                }
            }
#pragma unroll 4
            for (; i < ie; i += WI) {
                float av[V];
                load_a<float, float, V>(ap + i * Pp, av);
                const float bb = __ldg(bs + i);
#pragma unroll
                for (int v = 0; v < V; ++v) acc[v].fma_add(av[v], bb);
            }
        }
        if (WI > 1) {
            const uint32_t slot = wo * 32u + lane;
            if (wi > 0) {
                float* r = red + ((size_t)(wi - 1) * (WO * 32u) + slot) * (2 * V);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    r[2 * v] = acc[v].s;
                    r[2 * v + 1] = acc[v].c;
                }
            }
            __syncthreads();
            if (wi == 0) {
                for (uint32_t w = 1; w < (uint32_t)WI; ++w) {
                    const float* r = red + ((size_t)(w - 1) * (WO * 32u) + slot) * (2 * V);
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v].merge(r[2 * v], r[2 * v + 1]);
                }
            }
            __syncthreads();
        }
        if (wi == 0 && valid) {
            if (P.nseg == 1) {
#pragma unroll
                for (int v = 0; v < V; ++v) P.c[o0 + v] = acc[v].value();
            } else {
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    BPair pr;
                    pr.s = acc[v].s;
                    pr.c = KAHAN ? acc[v].c : 0.f;
                    part[P.part_off + seg * outputs + o0 + v] = pr;
                }
            }
        }
    }
}

// Column unit with narrow loads (V = 1: odd prefixes or A at an odd offset;
// V = 2: prefixes even but not a multiple of 4): each thread owns COL1_MO
// vectors of V outputs, 32 vectors apart, so each row puts COL1_MO
// independent coalesced warp loads in flight per thread; every vector walks
// its column with one running pointer (one 64-bit add per load), and blocks of
// TLIBG_BATCH_COL1_LOADS scalar (TLIBG_BATCH_COL2_LOADS 8-byte) loads -- then
// halves, quarters, single rows -- are issued before their products.  A vector
// past the end re-reads vector 0's column (its sums are never stored) instead
// of predicating every load.
#ifndef TLIBG_BATCH_COL1_LOADS
#define TLIBG_BATCH_COL1_LOADS 24
#endif
#ifndef TLIBG_BATCH_COL2_LOADS
#define TLIBG_BATCH_COL2_LOADS 16
#endif
template <int V> __device__ __forceinline__ void load_narrow(const float* p, float (&out)[V])
{
    if constexpr (V == 1) {
        out[0] = __ldcs(p);
    } else {
        const float2 t = __ldcs(reinterpret_cast<const float2*>(p));
        out[0] = t.x;
        out[1] = t.y;
    }
}

template <int UB, int V, bool KAHAN>
__device__ __forceinline__ void coln_rows(Acc<float, KAHAN> (&acc)[COL1_MO][V], const float* (&rp)[COL1_MO],
                                          uint64_t step, const float* __restrict__ bs, uint64_t i, uint32_t WI)
{
    float av[UB][COL1_MO][V];
#pragma unroll
    for (int u = 0; u < UB; ++u)
#pragma unroll
        for (int m = 0; m < COL1_MO; ++m) {
            load_narrow<V>(rp[m], av[u][m]);
            rp[m] += step;
        }
#pragma unroll
    for (int u = 0; u < UB; ++u) {
        const float bb = __ldg(bs + i + u * WI);
#pragma unroll
        for (int m = 0; m < COL1_MO; ++m)
#pragma unroll
            for (int v = 0; v < V; ++v) acc[m][v].fma_add(av[u][m][v], bb);
    }
}

template <int V, bool KAHAN>
__device__ __forceinline__ void coln_unit(const BProb& P, uint64_t lu, int WI, float* red, BPair* __restrict__ part)
{
    constexpr int MO = COL1_MO;
    constexpr int U = (V == 1 ? TLIBG_BATCH_COL1_LOADS : TLIBG_BATCH_COL2_LOADS) / MO;
    const uint32_t WO = (BLOCK / 32) / WI;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t wi = warp % WI, wo = warp / WI;
    const uint64_t TO = (uint64_t)WO * 32u * V * MO;
    const uint64_t outputs = P.S * P.P;
    const uint64_t seg = P.nseg == 1 ? 0 : idx_div(lu, P.tdiv);
    const uint64_t tile0 = (lu - seg * P.upseg) * P.tpu;
    const uint64_t tile1 = min(P.tiles, tile0 + P.tpu);
    const uint64_t ib = seg * P.seg_len;
    const uint64_t ie = min(P.nq, ib + P.seg_len);
    const uint64_t Pp = P.P, nq = P.nq;
    const float* __restrict__ A = P.a;
    const float* __restrict__ bs = P.b;
    const uint64_t step = (uint64_t)WI * Pp;

    for (uint64_t tile = tile0; tile < tile1; ++tile) {
        // vector m of this thread: outputs o0 + 32 V m .. + V - 1
        const uint64_t o0 = tile * TO + (uint64_t)wo * 32u * V * MO + (uint64_t)lane * V;
        bool ok[MO];
#pragma unroll
        for (int m = 0; m < MO; ++m) ok[m] = o0 + 32u * V * m < outputs;
        Acc<float, KAHAN> acc[MO][V];
#pragma unroll
        for (int m = 0; m < MO; ++m)
#pragma unroll
            for (int v = 0; v < V; ++v) acc[m][v].init();
        if (ok[0]) {
            const float* rp[MO];
#pragma unroll
            for (int m = 0; m < MO; ++m) {
                const uint64_t o = ok[m] ? o0 + 32u * V * m : o0;
                const uint64_t sl = idx_div(o, P.pdiv);
                rp[m] = A + (sl * nq + ib + wi) * Pp + (o - sl * Pp);
            }
            uint64_t i = ib + wi;
            for (; i + (U - 1) * WI < ie; i += U * WI) coln_rows<U, V>(acc, rp, step, bs, i, WI);
            if (i + (U / 2 - 1) * WI < ie) {
                coln_rows<U / 2, V>(acc, rp, step, bs, i, WI);
                i += (U / 2) * WI;
            }
            if (i + (U / 4 - 1) * WI < ie) {
                coln_rows<U / 4, V>(acc, rp, step, bs, i, WI);
                i += (U / 4) * WI;
            }
            for (; i < ie; i += WI) coln_rows<1, V>(acc, rp, step, bs, i, WI);
        }
        if (WI > 1) {
            const uint32_t slot = wo * 32u + lane;
            if (wi > 0) {
                float* r = red + ((size_t)(wi - 1) * (WO * 32u) + slot) * (2 * MO * V);
#pragma unroll
                for (int m = 0; m < MO; ++m)
#pragma unroll
                    for (int v = 0; v < V; ++v) {
                        r[2 * (m * V + v)] = acc[m][v].s;
                        r[2 * (m * V + v) + 1] = acc[m][v].c;
                    }
            }
            __syncthreads();
            if (wi == 0) {
                for (uint32_t w = 1; w < (uint32_t)WI; ++w) {
                    const float* r = red + ((size_t)(w - 1) * (WO * 32u) + slot) * (2 * MO * V);
#pragma unroll
                    for (int m = 0; m < MO; ++m)
#pragma unroll
                        for (int v = 0; v < V; ++v) acc[m][v].merge(r[2 * (m * V + v)], r[2 * (m * V + v) + 1]);
                }
            }
            __syncthreads();
        }
        if (wi == 0) {
#pragma unroll
            for (int m = 0; m < MO; ++m) {
                if (!ok[m]) continue;
                const uint64_t o = o0 + 32u * V * m;
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    if (P.nseg == 1) {
                        P.c[o + v] = acc[m][v].value();
                    } else {
                        BPair pr;
                        pr.s = acc[m][v].s;
                        pr.c = KAHAN ? acc[m][v].c : 0.f;
                        part[P.part_off + seg * outputs + o + v] = pr;
                    }
                }
            }
        }
    }
}

template <bool KAHAN>
__device__ __forceinline__ void combine_problem(const BProb& P, const BPair* __restrict__ part)
{
    const uint64_t outputs = P.S * P.P;
    for (uint64_t o = threadIdx.x; o < outputs; o += BLOCK) {
        const BPair* pp = part + P.part_off + o;
        float2 first = __ldcg(reinterpret_cast<const float2*>(pp));
        Acc<float, KAHAN> acc;
        acc.s = first.x;
        acc.c = first.y;
        for (uint32_t g = 1; g < P.nseg; ++g) {
            const float2 q = __ldcg(reinterpret_cast<const float2*>(pp + (uint64_t)g * outputs));
            acc.merge(q.x, q.y);
        }
        P.c[o] = acc.value();
    }
}

// Resident CTAs per SM the executor is compiled for (registers capped so that
// this many fit): more warps in flight per SM for the latency-bound units.
// Measured on GB300 (4096 uneven problems, fixed rule, atomic queue): 1 -> 6.1
// ms, 5 -> 3.9 ms, 6 -> 3.7 ms, 7 and 8 -> 3.5 ms per launch, despite spills;
// with two short rows per round in the row units 6, 7 and 8 all give
// 3.47-3.50 ms, 6 with the fewest spills.
#ifndef TLIBG_BATCH_MIN_CTAS
#define TLIBG_BATCH_MIN_CTAS 6
#endif

// Resident CTAs per SM the scalar-column executor is compiled for (more
// registers per thread than the generic one: its loads in flight).
#ifndef TLIBG_BATCH_COL1_MIN_CTAS
#define TLIBG_BATCH_COL1_MIN_CTAS 4
#endif
template <int CLS> __host__ __device__ constexpr int exec_min_ctas()
{
    return CLS == CLS_COL1 ? TLIBG_BATCH_COL1_MIN_CTAS : TLIBG_BATCH_MIN_CTAS;
}

// CTA loop over the class's units from its atomic queue: thread 0 claims the
// next unit one iteration ahead (the atomic's latency hidden by a whole unit)
// and reads its problem index; one CTA barrier per unit (two more for a split
// problem's completion count).  Units are large (TLIBG_BATCH_UNIT_BYTES of A)
// so the per-unit latency -- the claim, the problem's descriptor, the first
// loads' round trip -- is small next to a unit's streaming time.
template <bool KAHAN, int CLS>
__global__ void __launch_bounds__(BLOCK, exec_min_ctas<CLS>())
    batch_exec(BProb* __restrict__ pr, const uint32_t* __restrict__ unit_map, BCtl* ctl, BPair* __restrict__ part)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* red = reinterpret_cast<float*>(smem_raw);
    __shared__ unsigned long long s_unit;
    __shared__ int s_prob, s_last;
    const unsigned long long total = *reinterpret_cast<volatile unsigned long long*>(&ctl->total[CLS]);
    const int record = *reinterpret_cast<volatile int*>(&ctl->record);
    long long t_unit = 0;
    unsigned long long next = 0;
    if (threadIdx.x == 0) next = atomicAdd(&ctl->head[CLS], 1ull);

    while (true) {
        if (threadIdx.x == 0) {
            s_unit = next;
            if (next < total) {
                s_prob = (int)unit_map[next];
                next = atomicAdd(&ctl->head[CLS], 1ull);   // consumed on the next iteration
            }
        }
        __syncthreads();
        const unsigned long long u = s_unit;
        if (u >= total) break;
        if (record && threadIdx.x == 0) t_unit = clock64();
        const int pi = s_prob;
        const BProb& P = pr[pi];
        const uint64_t lu = u - P.unit_begin;
        if constexpr (CLS == CLS_COL1) {
            if (P.vec == 2) coln_unit<2, KAHAN>(P, lu, P.group, red, part);
            else coln_unit<1, KAHAN>(P, lu, P.group, red, part);
        } else if (P.kind == KIND_ROW) {
            switch (P.vec) {
            case 4: row_unit<4, KAHAN>(P, lu, P.group, part); break;
            case 2: row_unit<2, KAHAN>(P, lu, P.group, part); break;
            default: row_unit<1, KAHAN>(P, lu, P.group, part); break;
            }
        } else {
            col_unit<4, KAHAN>(P, lu, P.group, red, part);
        }
        if (P.nseg > 1) {
            __syncthreads();   // this CTA's partial stores are issued
            if (threadIdx.x == 0) {
                __threadfence();
                const unsigned int old = atomicAdd(&pr[pi].done, 1u);
                s_last = (old + 1u == P.units);
            }
            __syncthreads();
            if (s_last) {
                __threadfence();
                combine_problem<KAHAN>(P, part);
            }
        }
        __syncthreads();
        if (record && threadIdx.x == 0) atomicAdd(&pr[pi].cycles, (unsigned long long)(clock64() - t_unit));
    }
}

// --------------------------------------------------------------------------
// staged row units: one lane per row from shared memory (variant 8)
// --------------------------------------------------------------------------
// Every warp works alone, on units from the atomic queue; a unit is BRT_TPU
// tiles of 32 R consecutive rows of one problem (contiguous in HBM).  Each
// tile moves into the warp's two-stage ring with one TMA bulk copy (ragged
// head and tail by plain loads), the problem's b beside it; the warp then
// walks one row per lane from shared memory (even n_q from a lane-dependent
// column, so the lanes' reads spread over the banks) while the next tile is in
// flight.  Waits are bounded; an expired wait sets the batch error word and
// the warp leaves once its copies in flight have landed (bounded).
template <bool KAHAN>
__global__ void __launch_bounds__(BRT_THREADS) batch_rowtile(BProb* __restrict__ pr, const uint32_t* __restrict__ unit_map_r,
                                                             BCtl* ctl)
{
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw) + warp * BRT_NS;
    unsigned char* wbase = smem_raw + 128 + (size_t)warp * BRT_WARP_BYTES;
    float* barea = reinterpret_cast<float*>(wbase);                        // [BRT_NS][BRT_MAX_NQ]
    unsigned char* ring = wbase + (size_t)BRT_NS * BRT_MAX_NQ * 4;         // [BRT_NS][BRT_SLOT]
    if (lane == 0) {
        for (int s = 0; s < BRT_NS; ++s) mbar_init(full + s, 1);
        fence_mbar_init();
    }
    __syncwarp();
    const unsigned long long total = *reinterpret_cast<volatile unsigned long long*>(&ctl->total[CLS_STAGED]);
    const int record = *reinterpret_cast<volatile int*>(&ctl->record);

    // issue side: the problem and tile range of the unit being issued
    int iprob = -1;
    uint64_t it = 0, it_end = 0;
    auto advance = [&]() -> bool {
        while (it >= it_end) {
            unsigned long long v = 0;
            if (lane == 0) v = atomicAdd(&ctl->head[CLS_STAGED], 1ull);
            const unsigned long long u = __shfl_sync(0xffffffffu, v, 0);
            if (u >= total) return false;
            iprob = (int)__ldg(unit_map_r + u);
            const BProb& P = pr[iprob];
            const uint64_t R = brt_rows_per_lane(P.nq);
            const uint64_t tiles = (P.S + 32 * R - 1) / (32 * R);
            it = (u - P.unit_begin) * BRT_TPU;
            it_end = min(tiles, it + BRT_TPU);
        }
        return true;
    };
    int sprob[BRT_NS];
    uint64_t stile[BRT_NS];
    auto issue = [&](int s) {
        const BProb& P = pr[iprob];
        const uint32_t nq = (uint32_t)P.nq;
        const uint64_t R = brt_rows_per_lane(nq);
        const uint64_t r0 = it * 32 * R, r1 = min(P.S, r0 + 32 * R);
        for (uint32_t e = lane; e < nq; e += 32) barea[s * BRT_MAX_NQ + e] = __ldg(P.b + e);
        stream_issue<float>(P.a, r0 * nq, r1 * nq, ring + (size_t)s * BRT_SLOT, full + s, lane);
        sprob[s] = iprob;
        stile[s] = it;
        ++it;
    };
    bool more = advance();
    uint32_t issued = 0;
#pragma unroll
    for (int s = 0; s < BRT_NS; ++s)
        if (more) {
            issue(s);
            ++issued;
            more = advance();
        }
    for (uint32_t c = 0; c < issued; ++c) {
        const int s = (int)(c % BRT_NS);
        long long t0 = 0;
        if (record && lane == 0) t0 = clock64();
        const bool ok = mbar_wait_bounded(full + s, (c / BRT_NS) & 1u, &g_batch_error);
        if (__any_sync(0xffffffffu, !ok)) {
            // leave only after this warp's other copy in flight has landed (bounded)
            if (c + 1 < issued) mbar_wait_bounded(full + ((c + 1) % BRT_NS), ((c + 1) / BRT_NS) & 1u, &g_batch_error);
            return;
        }
        const int pi = sprob[s];
        const BProb& P = pr[pi];
        const uint32_t nq = (uint32_t)P.nq;
        const uint32_t R = brt_rows_per_lane(nq);
        const uint64_t r0 = stile[s] * 32 * R;
        const uint32_t mis = (uint32_t)(reinterpret_cast<uintptr_t>(P.a + r0 * nq) & 15u);
        const float* rows = reinterpret_cast<const float*>(ring + (size_t)s * BRT_SLOT + mis);
        const float* sb = barea + s * BRT_MAX_NQ;
        const uint32_t rot = (nq & 1u) ? 0u : lane % nq;
        float out[4];
        auto walk = [&](auto RC) {
            constexpr int RR = decltype(RC)::value;
            Acc<float, KAHAN> acc[RR];
#pragma unroll
            for (int r = 0; r < RR; ++r) acc[r].init();
            if (r0 + lane < P.S) {
                // rows lane + 32 r of the tile; one past the end re-reads row `lane`
                const float* rp[RR];
#pragma unroll
                for (int r = 0; r < RR; ++r)
                    rp[r] = rows + (size_t)((r0 + lane + 32u * r < P.S) ? lane + 32u * r : lane) * nq;
                rowt_dot_any<RR, false>(acc, rp, sb, (const float2*)nullptr, nq, rot);
            }
#pragma unroll
            for (int r = 0; r < RR; ++r) out[r] = acc[r].value();
        };
        if (R == 4) walk(std::integral_constant<int, 4>{});
        else if (R == 2) walk(std::integral_constant<int, 2>{});
        else walk(std::integral_constant<int, 1>{});
        __syncwarp();   // every lane is done with the stage
        float* C = P.c;
        const uint64_t S = P.S;
        if (more) {
            issue(s);
            ++issued;
            more = advance();
        }
        for (uint32_t r = 0; r < R; ++r) {
            const uint64_t row = r0 + lane + 32u * r;
            if (row < S) C[row] = out[r];
        }
        if (record && lane == 0) atomicAdd(&pr[pi].cycles, (unsigned long long)(clock64() - t0));
    }
}

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------
namespace {

std::mutex g_model_mu;
std::vector<float> g_model;   // installed cost-model parameters (empty: none)
float g_model_margin = 0.f;   // minimum predicted relative gain to leave the fixed rule

size_t exec_smem_bytes()
{
    const size_t red_floats = (size_t)(8 - 1) * 1 * 32 * 2 * 4;   // largest: WI = 8, V = 4
    return red_floats * 4;
}

// Resident CTAs per SM of a class's executor kernel (its launch grid is SMs x this).
const void* exec_fn(bool kahan, int cls)
{
    if (cls == CLS_COL1)
        return kahan ? reinterpret_cast<const void*>(batch_exec<true, CLS_COL1>)
                     : reinterpret_cast<const void*>(batch_exec<false, CLS_COL1>);
    return kahan ? reinterpret_cast<const void*>(batch_exec<true, CLS_GENERIC>)
                 : reinterpret_cast<const void*>(batch_exec<false, CLS_GENERIC>);
}

int exec_ctas_per_sm(bool kahan, int cls)
{
    static int cache[2][2] = {{-1, -1}, {-1, -1}};
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    int& c = cache[kahan ? 1 : 0][cls == CLS_COL1 ? 1 : 0];
    if (c >= 0) return c;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, exec_fn(kahan, cls), BLOCK, exec_smem_bytes()) != cudaSuccess) {
        cudaGetLastError();
        n = 1;
    }
    c = std::max(1, n);
    return c;
}

int rowtile_ctas_per_sm(bool kahan)
{
    static int cache[2] = {-1, -1};
    static std::mutex mu;
    std::lock_guard<std::mutex> lk(mu);
    int& c = cache[kahan ? 1 : 0];
    if (c >= 0) return c;
    const void* fn = kahan ? reinterpret_cast<const void*>(batch_rowtile<true>)
                           : reinterpret_cast<const void*>(batch_rowtile<false>);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)BRT_SMEM);
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, BRT_THREADS, BRT_SMEM) != cudaSuccess) {
        cudaGetLastError();
        n = 1;
    }
    c = std::max(1, n);
    return c;
}

// widest load (elements) the layout and the pointers' alignment allow
int batch_vec(int kind, const CanonView& cn, const void* a, const void* b)
{
    int vec = 4;
    while (vec > 1 && !((kind == KIND_ROW ? cn.nq : cn.P) % vec == 0 &&
                        (reinterpret_cast<uintptr_t>(a) % (vec * 4)) == 0 &&
                        (kind == KIND_COL || (reinterpret_cast<uintptr_t>(b) % (vec * 4)) == 0)))
        vec /= 2;
    return vec;
}

// The fixed rule the engine uses without the cost model: the best single
// variant of each (kernel family, widest load, short row) class, re-derived
// from the autotuner's data (ttv_gb300/data/tuning_db.npz, 20,000 training
// shapes timed with every variant inside mixed batches; costmodel.py
// derive_fixed_rule): q-fastest rows of at most 64 elements staged through
// shared memory (variant 8), longer rows two lanes per row (variant 2),
// column problems one warp row per tile and no split (variant 0), for every
// load width.  Its aggregate time on held-out shapes is 2.5 % above
// exhaustive tuning's.
constexpr int FIXED_RULE[2][3][2] = {
    // [kind][vec 1, 2, 4][long row, short row]
    {{2, 8}, {2, 8}, {2, 8}},   // row form
    {{0, 0}, {0, 0}, {0, 0}},   // column form
};
int heuristic_variant(int kind, uint64_t P, uint64_t nq, uint64_t S, int vec)
{
    (void)P;
    (void)S;
    const int vi = vec >= 4 ? 2 : (vec == 2 ? 1 : 0);
    const int shrt = (kind == KIND_ROW && nq <= (uint64_t)BRT_MAX_NQ) ? 1 : 0;
    return FIXED_RULE[kind == KIND_ROW ? 0 : 1][vi][shrt];
}

}  // namespace
}  // namespace tlibg

using namespace tlibg;

struct tlibg_batch {
    int count = 0;
    int select = TLIBG_SELECT_HEURISTIC;
    int fixed_variant = 0;
    bool kahan = true;
    int grid[NCLS] = {0, 0, 0};    // CTAs of each class's kernel
    int slots[NCLS] = {1, 1, 1};   // resident CTAs (staged rows: warps) per SM of each class
    BProb* d_prob = nullptr;
    BCtl* d_ctl = nullptr;
    uint32_t* d_map[NCLS] = {nullptr, nullptr, nullptr};   // unit -> problem of each class
    BPair* d_part = nullptr;
    float* d_model = nullptr;
    float log2_count = 0.f;
    float log2_keep = 0.f;   // log2(1 - margin)
    bool planned = false;          // the plan kernels ran for the current variants
    cudaStream_t side[2] = {nullptr, nullptr};      // the scalar-column and staged-row kernels' streams
    cudaEvent_t ev_fork = nullptr, ev_join[2] = {nullptr, nullptr};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace {

// The plan (variants -> units, queues, unit maps) runs once per variant set:
// at creation and after a forced variant changes; every launch then only
// resets the queues and counters and runs the class kernels.
int enqueue_plan(tlibg_batch* bt, cudaStream_t st)
{
    uint64_t n = 0;
    if (bt->select == TLIBG_SELECT_FIXED) {
        batch_set_variant<<<(bt->count + 255) / 256, 256, 0, st>>>(bt->d_prob, bt->count, bt->fixed_variant);
        ++n;
    }
    batch_plan<<<1, 1024, 0, st>>>(bt->d_prob, bt->count, bt->d_ctl);
    batch_fill_maps<<<(bt->count + 7) / 8, 256, 0, st>>>(bt->d_prob, bt->count, bt->d_map[0], bt->d_map[1],
                                                        bt->d_map[2]);
    n += 2;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return internal_cuda_fail(e, "batch plan");
    internal_count_launches(n);
    bt->planned = true;
    return TLIBG_OK;
}

int enqueue(tlibg_batch* bt, cudaStream_t st)
{
    if (!bt->planned) {
        const int s = enqueue_plan(bt, st);
        if (s) return s;
    }
    batch_reset<<<(bt->count + 255) / 256, 256, 0, st>>>(bt->d_prob, bt->count, bt->d_ctl);
    // The class kernels are independent: the scalar-column and staged-row
    // kernels go on two side streams forked from `st` (branches of the CUDA
    // graph), so each one's CTAs fill the SMs the others' last units leave.
    const size_t smem = exec_smem_bytes();
    cudaEventRecord(bt->ev_fork, st);
    cudaStreamWaitEvent(bt->side[0], bt->ev_fork, 0);
    cudaStreamWaitEvent(bt->side[1], bt->ev_fork, 0);
    if (bt->kahan) {
        batch_exec<true, CLS_GENERIC><<<bt->grid[0], BLOCK, smem, st>>>(bt->d_prob, bt->d_map[0], bt->d_ctl, bt->d_part);
        batch_exec<true, CLS_COL1><<<bt->grid[1], BLOCK, smem, bt->side[0]>>>(bt->d_prob, bt->d_map[1], bt->d_ctl, bt->d_part);
        batch_rowtile<true><<<bt->grid[2], BRT_THREADS, BRT_SMEM, bt->side[1]>>>(bt->d_prob, bt->d_map[2], bt->d_ctl);
    } else {
        batch_exec<false, CLS_GENERIC><<<bt->grid[0], BLOCK, smem, st>>>(bt->d_prob, bt->d_map[0], bt->d_ctl, bt->d_part);
        batch_exec<false, CLS_COL1><<<bt->grid[1], BLOCK, smem, bt->side[0]>>>(bt->d_prob, bt->d_map[1], bt->d_ctl, bt->d_part);
        batch_rowtile<false><<<bt->grid[2], BRT_THREADS, BRT_SMEM, bt->side[1]>>>(bt->d_prob, bt->d_map[2], bt->d_ctl);
    }
    cudaEventRecord(bt->ev_join[0], bt->side[0]);
    cudaEventRecord(bt->ev_join[1], bt->side[1]);
    cudaStreamWaitEvent(st, bt->ev_join[0], 0);
    cudaStreamWaitEvent(st, bt->ev_join[1], 0);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return internal_cuda_fail(e, "batch launch");
    internal_count_launches(1 + NCLS);
    return TLIBG_OK;
}

int launches_per_run(const tlibg_batch* bt)
{
    return 1 + NCLS;   // reset + the class kernels (the plan is not part of a launch)
}

void release(tlibg_batch* bt)
{
    if (!bt) return;
    if (bt->exec) cudaGraphExecDestroy(bt->exec);
    if (bt->graph) cudaGraphDestroy(bt->graph);
    for (int i = 0; i < 2; ++i) {
        if (bt->side[i]) cudaStreamDestroy(bt->side[i]);
        if (bt->ev_join[i]) cudaEventDestroy(bt->ev_join[i]);
    }
    if (bt->ev_fork) cudaEventDestroy(bt->ev_fork);
    if (bt->d_prob) cudaFree(bt->d_prob);
    if (bt->d_ctl) cudaFree(bt->d_ctl);
    for (int c = 0; c < NCLS; ++c)
        if (bt->d_map[c]) cudaFree(bt->d_map[c]);
    if (bt->d_part) cudaFree(bt->d_part);
    if (bt->d_model) cudaFree(bt->d_model);
    delete bt;
}

int create_fail(tlibg_batch* bt, int code, const std::string& msg)
{
    release(bt);
    return internal_fail(code, msg);
}

}  // namespace

extern "C" {

int tlibg_set_cost_model(const float* params, size_t count, float margin)
{
    std::lock_guard<std::mutex> lk(g_model_mu);
    if (!params) {
        g_model.clear();
        return internal_ok();
    }
    if (!(margin >= 0.f && margin < 1.f))
        return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_set_cost_model: margin must be in [0, 1)");
    g_model_margin = margin;
    if (count != (size_t)MLP_PARAMS)
        return internal_fail(TLIBG_ERR_ARGUMENT,
                             "tlibg_set_cost_model: expected " + std::to_string(MLP_PARAMS) + " parameters");
    g_model.assign(params, params + count);
    return internal_ok();
}

int tlibg_batch_features(const tlibg_problem* pr, size_t count, float* feat, int* kind, int* heuristic)
{
    if ((!pr || !feat) && count) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_batch_features: null argument");
    for (size_t i = 0; i < count; ++i) {
        const tlibg_problem& x = pr[i];
        CanonView cn;
        const int st = internal_analyse(x.q, x.p, x.a, x.na, x.wa, x.pia, x.b, x.nb, x.c, x.nc, x.wc, x.pic, &cn);
        if (st) return st;
        if ((reinterpret_cast<uintptr_t>(x.a) | reinterpret_cast<uintptr_t>(x.b) | reinterpret_cast<uintptr_t>(x.c)) & 3u)
            return internal_fail(TLIBG_ERR_UNSUPPORTED, "tlibg: a, b and c must be aligned to their element sizes");
        size_t k = 0;
        while (x.pia[k] != x.q) ++k;
        float* f = feat + i * NFEAT;
        f[0] = (float)x.p / 8.f;
        f[1] = x.p > 1 ? (float)k / (float)(x.p - 1) : 0.f;
        f[2] = (float)std::log2((double)cn.P) / 24.f;
        f[3] = (float)std::log2((double)cn.nq) / 24.f;
        f[4] = (float)std::log2((double)cn.S) / 24.f;
        f[5] = 0.f;   // fp32
        f[6] = (float)std::log2((double)count) / 16.f;
        const int kd = cn.P == 1 ? KIND_ROW : KIND_COL;
        f[7] = (float)batch_vec(kd, cn, x.a, x.b) / 4.f;   // widest legal load (alignment)
        if (kind) kind[i] = kd;
        if (heuristic) heuristic[i] = heuristic_variant(kd, cn.P, cn.nq, cn.S, batch_vec(kd, cn, x.a, x.b));
    }
    return internal_ok();
}

int tlibg_batch_create(int dtype, const tlibg_problem* probs, size_t count, const tlibg_batch_options* opt,
                       void* stream, tlibg_batch** out)
{
    if (!out) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_batch_create: null output handle");
    *out = nullptr;
    if (dtype != TLIBG_F32)
        return internal_fail(TLIBG_ERR_UNSUPPORTED, "tlibg_batch_create: batches are fp32 (TLIBG_F32)");
    if (!probs || count == 0 || count > ((size_t)1 << 24))
        return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_batch_create: need 1 to 2^24 problems");
    const int sms = internal_sms();
    if (!sms) return internal_fail(TLIBG_ERR_CUDA, "tlibg: no usable CUDA device");
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    tlibg_batch* bt = new tlibg_batch();
    bt->count = (int)count;
    bt->select = opt ? opt->select : TLIBG_SELECT_HEURISTIC;
    bt->fixed_variant = opt ? opt->variant : 0;
    bt->kahan = !(opt && opt->accumulate == TLIBG_ACC_PLAIN);
    const bool use_graph = !(opt && opt->no_graph);
    const bool have_given = opt && opt->variants;
    bt->log2_count = (float)std::log2((double)count);
    if (bt->select < TLIBG_SELECT_HEURISTIC || bt->select > TLIBG_SELECT_GIVEN)
        return create_fail(bt, TLIBG_ERR_ARGUMENT, "tlibg_batch_create: unknown selection mode");
    if (bt->select == TLIBG_SELECT_FIXED && (bt->fixed_variant < 0 || bt->fixed_variant >= NVARIANT))
        return create_fail(bt, TLIBG_ERR_ARGUMENT,
                           "tlibg_batch_create: variant must be in 0.." + std::to_string(NVARIANT - 1));

    std::vector<float> feat(count * NFEAT);
    std::vector<int> kinds(count), heur(count);
    int s = tlibg_batch_features(probs, count, feat.data(), kinds.data(), heur.data());
    if (s) {
        release(bt);
        return s;
    }
    std::vector<float> model;
    if (bt->select == TLIBG_SELECT_LEARNED) {
        std::lock_guard<std::mutex> lk(g_model_mu);
        model = g_model;
        bt->log2_keep = (float)std::log2(1.0 - (double)g_model_margin);
    }
    if (bt->select == TLIBG_SELECT_LEARNED && model.empty())
        // no model installed: exhaustive-tuning results when given, else the fixed rule
        bt->select = have_given ? TLIBG_SELECT_GIVEN : TLIBG_SELECT_HEURISTIC;
    if (bt->select == TLIBG_SELECT_GIVEN && !have_given)
        return create_fail(bt, TLIBG_ERR_ARGUMENT, "tlibg_batch_create: TLIBG_SELECT_GIVEN needs variants");

    // descriptors; unit map and partial scratch sized for the worst variant of each problem
    std::vector<BProb> hp(count);
    uint64_t total_units[NCLS] = {0, 0, 0}, max_part = 0;
    for (size_t i = 0; i < count; ++i) {
        const tlibg_problem& x = probs[i];
        s = internal_check_device_pointers(x.a, x.b, x.c);
        if (s) {
            release(bt);
            return s;
        }
        CanonView cn;
        internal_analyse(x.q, x.p, x.a, x.na, x.wa, x.pia, x.b, x.nb, x.c, x.nc, x.wc, x.pic, &cn);
        BProb& b = hp[i];
        std::memset(&b, 0, sizeof(b));
        b.a = static_cast<const float*>(x.a);
        b.b = static_cast<const float*>(x.b);
        b.c = static_cast<float*>(x.c);
        b.P = cn.P;
        b.nq = cn.nq;
        b.S = cn.S;
        b.kind = kinds[i];
        b.vec = batch_vec(b.kind, cn, x.a, x.b);
        std::copy(feat.begin() + i * NFEAT, feat.begin() + (i + 1) * NFEAT, b.feat);
        // the staged row variant takes short q-fastest rows only
        b.valid_mask = (1u << NVARIANT) - 1u;
        if (!(b.kind == KIND_ROW && b.nq <= (uint64_t)BRT_MAX_NQ)) b.valid_mask &= ~(1u << VARIANT_STAGED);
        b.variant = heur[i];
        b.heuristic = heur[i];
        if (bt->select == TLIBG_SELECT_GIVEN) {
            const int v = opt->variants[i];
            if (v < 0 || v >= NVARIANT)
                return create_fail(bt, TLIBG_ERR_ARGUMENT,
                                   "tlibg_batch_create: variants must be in 0.." + std::to_string(NVARIANT - 1));
            b.variant = v;
        }
        uint64_t mu = 0, mp = 0;
        for (int v = 0; v < NVARIANT; ++v) {
            if (v == VARIANT_STAGED) continue;
            int g;
            uint32_t ns;
            decode_variant(b.kind, v, b.nq, &g, &ns);
            uint64_t sl;
            mu = std::max(mu, unit_count(b.kind, g, b.vec, b.P, b.nq, b.S, ns, &sl));
            const uint64_t nsr = (b.nq + sl - 1) / sl;
            if (nsr > 1) mp = std::max(mp, nsr * b.S * b.P);
        }
        // units in the class the problem runs in unless staged (its kind and load width
        // decide), and in the staged class where that variant applies
        total_units[(b.kind == KIND_COL && b.vec <= 2) ? CLS_COL1 : CLS_GENERIC] += mu;
        max_part += mp;
        if ((b.valid_mask >> VARIANT_STAGED) & 1u) total_units[CLS_STAGED] += brt_units(b.nq, b.S);
    }
    bt->slots[CLS_GENERIC] = exec_ctas_per_sm(bt->kahan, CLS_GENERIC);
    bt->slots[CLS_COL1] = exec_ctas_per_sm(bt->kahan, CLS_COL1);
    bt->slots[CLS_STAGED] = rowtile_ctas_per_sm(bt->kahan) * BRT_WARPS;
    bt->grid[CLS_GENERIC] = sms * bt->slots[CLS_GENERIC];
    bt->grid[CLS_COL1] = sms * bt->slots[CLS_COL1];
    bt->grid[CLS_STAGED] = sms * (bt->slots[CLS_STAGED] / BRT_WARPS);
    for (int c = 0; c < NCLS; ++c)
        if (total_units[c] >= ((uint64_t)1 << 32))
            return create_fail(bt, TLIBG_ERR_UNSUPPORTED, "tlibg_batch_create: more than 2^32 work units");

    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) {
        if ((e = cudaStreamCreateWithFlags(&bt->side[i], cudaStreamNonBlocking)) == cudaSuccess)
            e = cudaEventCreateWithFlags(&bt->ev_join[i], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bt->ev_fork, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        release(bt);
        return internal_cuda_fail(e, "tlibg_batch_create: streams");
    }
    if ((e = internal_malloc((void**)&bt->d_prob, count * sizeof(BProb))) != cudaSuccess ||
        (e = internal_malloc((void**)&bt->d_ctl, sizeof(BCtl))) != cudaSuccess ||
        (e = internal_malloc((void**)&bt->d_map[0], std::max<uint64_t>(total_units[0], 1) * sizeof(uint32_t))) != cudaSuccess ||
        (e = internal_malloc((void**)&bt->d_map[1], std::max<uint64_t>(total_units[1], 1) * sizeof(uint32_t))) != cudaSuccess ||
        (e = internal_malloc((void**)&bt->d_map[2], std::max<uint64_t>(total_units[2], 1) * sizeof(uint32_t))) != cudaSuccess ||
        (e = internal_malloc((void**)&bt->d_part, std::max<uint64_t>(max_part, 1) * sizeof(BPair))) != cudaSuccess ||
        (!model.empty() && (e = internal_malloc((void**)&bt->d_model, MLP_PARAMS * sizeof(float))) != cudaSuccess)) {
        cudaGetLastError();
        return create_fail(bt, TLIBG_ERR_NOMEM, std::string("tlibg_batch_create: ") + cudaGetErrorString(e));
    }
    cudaMemcpyAsync(bt->d_prob, hp.data(), count * sizeof(BProb), cudaMemcpyHostToDevice, st);
    BCtl hctl{};
    hctl.record = (opt && opt->record_costs) ? 1 : 0;
    cudaMemcpyAsync(bt->d_ctl, &hctl, sizeof(BCtl), cudaMemcpyHostToDevice, st);
    if (!model.empty() && bt->select == TLIBG_SELECT_LEARNED)
        cudaMemcpyAsync(bt->d_model, model.data(), MLP_PARAMS * sizeof(float), cudaMemcpyHostToDevice, st);
    if (bt->select == TLIBG_SELECT_LEARNED) {
        // the scores depend only on the descriptors and the model: select once,
        // every launch replays plan + exec with the chosen variants
        const int threads = bt->count * SELECT_LANES;
        batch_select<<<(threads + 255) / 256, 256, 0, st>>>(bt->d_prob, bt->count, bt->d_model, bt->log2_count,
                                                            bt->log2_keep);
        internal_count_launches(1);
        if ((e = cudaGetLastError()) != cudaSuccess) {
            release(bt);
            return internal_cuda_fail(e, "batch select");
        }
    }
    // the plan runs once here (graph launches replay only reset + class kernels)
    if ((s = enqueue_plan(bt, st))) {
        release(bt);
        return s;
    }
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) {
        release(bt);
        return internal_cuda_fail(e, "tlibg_batch_create");
    }
    if (use_graph) {
        cudaStream_t cap = nullptr;
        if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)) != cudaSuccess) {
            release(bt);
            return internal_cuda_fail(e, "capture stream");
        }
        e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            s = enqueue(bt, cap);
            cudaGraph_t g = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(cap, &g);
            if (!s && e2 == cudaSuccess) {
                bt->graph = g;
                e = cudaGraphInstantiate(&bt->exec, g, 0);
            } else {
                e = e2 != cudaSuccess ? e2 : cudaErrorUnknown;
                if (g) cudaGraphDestroy(g);
            }
        }
        cudaStreamDestroy(cap);
        if (s) {
            release(bt);
            return s;
        }
        if (e != cudaSuccess) {
            release(bt);
            return internal_cuda_fail(e, "graph capture");
        }
    }
    *out = bt;
    return internal_ok();
}

int tlibg_batch_launch(tlibg_batch* bt, void* stream)
{
    NvtxRange nvtx("tlibg_batch_launch");
    if (!bt) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_batch_launch: null batch");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (bt->exec) {
        const cudaError_t e = cudaGraphLaunch(bt->exec, st);
        if (e != cudaSuccess) return internal_cuda_fail(e, "graph launch");
        internal_count_launches((uint64_t)launches_per_run(bt));
        return internal_ok();
    }
    const int s = enqueue(bt, st);
    return s ? s : internal_ok();
}

int tlibg_batch_set_variant(tlibg_batch* bt, int variant)
{
    if (!bt) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_batch_set_variant: null batch");
    if (bt->select != TLIBG_SELECT_FIXED || bt->exec)
        return internal_fail(TLIBG_ERR_ARGUMENT,
                             "tlibg_batch_set_variant: only for TLIBG_SELECT_FIXED batches built with no_graph");
    if (variant < 0 || variant >= NVARIANT)
        return internal_fail(TLIBG_ERR_ARGUMENT,
                             "tlibg_batch_set_variant: variant must be in 0.." + std::to_string(NVARIANT - 1));
    if (bt->fixed_variant != variant) bt->planned = false;
    bt->fixed_variant = variant;
    return internal_ok();
}

int tlibg_batch_variants(tlibg_batch* bt, int* out, void* stream)
{
    if (!bt || !out) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_batch_variants: null argument");
    std::vector<BProb> hp(bt->count);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(hp.data(), bt->d_prob, bt->count * sizeof(BProb), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return internal_cuda_fail(e, "tlibg_batch_variants");
    for (int i = 0; i < bt->count; ++i) out[i] = hp[i].variant;
    return internal_ok();
}

int tlibg_batch_costs(tlibg_batch* bt, uint64_t* cycles, void* stream)
{
    if (!bt || !cycles) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_batch_costs: null argument");
    std::vector<BProb> hp(bt->count);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaError_t e = cudaMemcpyAsync(hp.data(), bt->d_prob, bt->count * sizeof(BProb), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return internal_cuda_fail(e, "tlibg_batch_costs");
    // SM cycles: a unit's CTA (or, staged, warp) cycles over the CTAs (warps) resident per SM
    for (int i = 0; i < bt->count; ++i) {
        const uint64_t sl = (uint64_t)bt->slots[hp[i].cls];
        cycles[i] = (hp[i].cycles + sl / 2) / sl;
    }
    return internal_ok();
}

int tlibg_batch_destroy(tlibg_batch* bt)
{
    if (bt) {
        cudaDeviceSynchronize();
        release(bt);
    }
    return internal_ok();
}

int tlibg_ttv_batch(int dtype, const tlibg_problem* probs, size_t count, const tlibg_batch_options* opt,
                    void* stream)
{
    tlibg_batch* bt = nullptr;
    tlibg_batch_options o{};
    if (opt) o = *opt;
    o.no_graph = 1;   // one launch: nothing to replay
    int s = tlibg_batch_create(dtype, probs, count, &o, stream, &bt);
    if (s) return s;
    s = tlibg_batch_launch(bt, stream);
    cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    release(bt);
    return s;
}

int tlibg_ttv_batch_f32(const tlibg_problem* probs, int n, void* stream)
{
    if (n < 0) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_ttv_batch_f32: negative problem count");
    tlibg_batch_options o{};
    o.select = TLIBG_SELECT_LEARNED;   // the installed cost model, else the fixed rule
    return tlibg_ttv_batch(TLIBG_F32, probs, (size_t)n, &o, stream);
}

int tlibg_ttv_percall(int dtype, const tlibg_problem* probs, size_t count, void* stream)
{
    if (!probs && count) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_ttv_percall: null problems");
    for (size_t i = 0; i < count; ++i) {
        const tlibg_problem& x = probs[i];
        const int s = tlibg_ttv_ex(dtype, x.q, x.p, x.a, x.na, x.wa, x.pia, x.b, x.nb, x.c, x.nc, x.wc, x.pic,
                                   nullptr, stream);
        if (s) return s;
    }
    return internal_ok();
}

unsigned int tlibg_batch_device_error(void)
{
    unsigned int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_batch_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
    cudaMemcpyToSymbol(g_batch_error, &zero, sizeof(zero));
    return v;
}

}  // extern "C"
