// TMA-streamed TTV kernel (included by ttv_kernels.cu).
//
// A is read as NR rows of L contiguous elements:
//   row form    (P == 1):  NR = S,        L = n_q,  C[r]       = sum_k A[r, k] b[k]
//   column form (P >  1):  NR = S * n_q,  L = P,    C[s, j]   += A[s*n_q + i, j] b[i]
// Each CTA owns a static sequence of chunks (runs of whole rows, at most
// STREAM_STAGE bytes, contiguous in HBM).  Warp 0 is the producer: lane 0
// moves the 16-byte-aligned body of each chunk with one cp.async.bulk into a
// ring of STREAM_NS shared-memory stages (full barrier: transaction bytes),
// lanes 0-31 fetch the ragged head and tail (under 16 bytes each) with plain
// loads.  Warps 1..8 consume: they wait on the stage's full barrier, compute
// from shared memory, and release the stage on its empty barrier.  The ring,
// not registers, sets the bytes in flight, and row alignment does not matter.
// Every wait is bounded; an expired wait sets the device error word and the
// CTA leaves.
#pragma once

#include "ttv_rowwalk.cuh"

namespace tlibg {

constexpr int STREAM_STAGE = STREAM_STAGE_BYTES;   // bytes of A per chunk
constexpr int STREAM_NS = 4;                  // stages in the ring
constexpr int STREAM_NCW = 8;                 // consumer warps
constexpr int STREAM_NT = STREAM_NCW * 32;    // consumer threads
static_assert(STREAM_NT == STREAM_CONSUMERS, "consumer thread count");
constexpr int STREAM_THREADS = STREAM_NT + 32;
constexpr int STREAM_SLOT = STREAM_STAGE + 32;
constexpr int STREAM_MAXJ = 8;                // column form: outputs per consumer thread

struct SArgs {
    const void* a;
    const void* b;
    void* out;
    void* partial;
    uint64_t S, nq, P;
    uint64_t L;              // row length in elements
    uint64_t R;              // rows per chunk
    uint64_t units;          // row form: rows; column form: items (s, segment)
    uint64_t units_per_cta;
    uint64_t seg_len;        // column form: rows of a segment
    uint32_t nseg;
    uint32_t G;              // row form: lanes per row
    uint32_t RG;             // column form: row groups (P < consumer threads)
    uint32_t J;              // column form: outputs per thread (RG == 1)
};

// Chunk sequence of one CTA: a chunk is rows [r0, r1) of the NR x L view.
struct ChunkWalk {
    // column form: current item and the row range inside it
    uint64_t unit, unit_end;
    uint64_t r, r_end;   // row cursor and end of the current unit (global rows)
    __device__ __forceinline__ void begin(const SArgs& k, bool col)
    {
        unit = (uint64_t)blockIdx.x * k.units_per_cta;
        unit_end = min(k.units, unit + k.units_per_cta);
        if (col) {
            set_item(k);
        } else {
            r = unit;
            r_end = unit_end;
        }
    }
    __device__ __forceinline__ void set_item(const SArgs& k)
    {
        if (unit >= unit_end) {
            r = r_end = 0;
            return;
        }
        const uint64_t s = unit / k.nseg, seg = unit - s * k.nseg;
        const uint64_t i0 = seg * k.seg_len;
        const uint64_t i1 = min(k.nq, i0 + k.seg_len);
        r = s * k.nq + i0;
        r_end = s * k.nq + i1;
    }
    // next chunk [r0, r1); returns false when the CTA's sequence is exhausted.
    // `item_done` reports that the chunk ends its item (column form).
    __device__ __forceinline__ bool next(const SArgs& k, bool col, uint64_t& r0, uint64_t& r1,
                                         bool& item_done)
    {
        if (col) {
            while (r >= r_end) {
                if (unit >= unit_end) return false;
                ++unit;
                set_item(k);
                if (unit >= unit_end) return false;
            }
        } else if (r >= r_end) {
            return false;
        }
        r0 = r;
        r1 = min(r_end, r + k.R);
        r = r1;
        item_done = (r >= r_end);
        return true;
    }
};

__device__ __forceinline__ void consumer_sync() { asm volatile("bar.sync 1, %0;" ::"n"(STREAM_NT) : "memory"); }

template <typename TA, typename T, bool KAHAN, bool COL>
__global__ void __launch_bounds__(STREAM_THREADS) stream_kernel(SArgs k)
{
    pdl_prologue();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* empty = full + STREAM_NS;
    int* abort_flag = reinterpret_cast<int*>(empty + STREAM_NS);
    unsigned char* ring = smem_raw + 128;
    T* sbuf = reinterpret_cast<T*>(ring + STREAM_NS * STREAM_SLOT);   // row form: b; column form: reduction
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ Bv = static_cast<const T*>(k.b);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STREAM_NS; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, STREAM_NCW);
        }
        *abort_flag = 0;
        fence_mbar_init();
    }
    if (!COL && warp > 0) {
        // row form: the whole b in shared memory (L elements)
        for (uint64_t e = threadIdx.x - 32; e < k.L; e += STREAM_NT) sbuf[e] = Bv[e];
    }
    __syncthreads();

    if (warp == 0) {
        // ---------------- producer ----------------
        ChunkWalk w;
        w.begin(k, COL);
        uint64_t r0, r1;
        bool done;
        uint32_t c = 0;
        while (w.next(k, COL, r0, r1, done)) {
            const uint32_t slot = c % STREAM_NS;
            if (c >= (uint32_t)STREAM_NS) {
                const bool ok = mbar_wait_bounded(empty + slot, ((c / STREAM_NS) - 1) & 1u, &g_device_error);
                if (__any_sync(0xffffffffu, !ok)) {
                    if (lane == 0) *abort_flag = 1;
                    break;
                }
            }
            stream_issue<TA>(A, r0 * k.L, r1 * k.L, ring + slot * STREAM_SLOT, full + slot, lane);
            ++c;
        }
        return;
    }

    // ---------------- consumers ----------------
    const uint32_t ct = threadIdx.x - 32;   // consumer thread 0..255
    ChunkWalk w;
    w.begin(k, COL);
    uint64_t r0, r1;
    bool item_done;
    uint32_t c = 0;
    if (!COL) {
        const uint32_t G = k.G;
        const uint32_t gl = lane & (G - 1);
        const uint32_t grp = ct / G;               // group index in the CTA
        const uint32_t ngrp = STREAM_NT / G;
        while (w.next(k, COL, r0, r1, item_done)) {
            const uint32_t slot = c % STREAM_NS;
            const bool ok = mbar_wait_bounded(full + slot, (c / STREAM_NS) & 1u, &g_device_error);
            if (__any_sync(0xffffffffu, !ok)) return;   // no CTA-wide barrier follows in this form
            const unsigned char* base = ring + slot * STREAM_SLOT;
            const uint32_t mis = (uint32_t)(reinterpret_cast<uintptr_t>(A + r0 * k.L) & 15u);
            const TA* rows = reinterpret_cast<const TA*>(base + mis);
            const uint64_t nrows = r1 - r0;
            for (uint64_t rb = 0; rb < nrows; rb += ngrp) {   // warp-uniform trip count
                const uint64_t rr = rb + grp;
                const bool valid = rr < nrows;
                typename AccSel<T, KAHAN>::type acc;
                acc.init();
                if (valid) {
                    // Power-of-two rows: each group starts at a row-dependent offset (a
                    // multiple of G) and wraps, so groups reading rows a power of two apart
                    // do not share shared-memory banks.  Other lengths walk straight.
                    const TA* rp = rows + rr * k.L;
                    const uint32_t Lr = (uint32_t)k.L;
                    const uint32_t rot = (Lr & (Lr - 1)) == 0 ? (uint32_t)((rr * G) & (Lr - 1)) : 0u;
                    for (uint32_t e = rot + gl; e < Lr; e += G) acc.fma_add(Cvt<TA, T>::f(rp[e]), sbuf[e]);
                    for (uint32_t e = gl; e < rot; e += G) acc.fma_add(Cvt<TA, T>::f(rp[e]), sbuf[e]);
                }
                acc.fold();
                for (uint32_t off = G >> 1; off > 0; off >>= 1) {
                    const T os = __shfl_xor_sync(0xffffffffu, acc.s, off);
                    const T oc = __shfl_xor_sync(0xffffffffu, acc.c, off);
                    acc.merge(os, oc);
                }
                if (valid && gl == 0) static_cast<T*>(k.out)[r0 + rr] = acc.value();
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(empty + slot);
            ++c;
        }
        return;
    }

    // column form
    const uint32_t RG = k.RG, J = k.J;
    const uint64_t P = k.P;
    const uint32_t rg = RG > 1 ? ct / (uint32_t)P : 0;
    const uint32_t j0 = RG > 1 ? ct % (uint32_t)P : ct;
    const bool active = RG > 1 ? (ct < RG * (uint32_t)P) : true;
    typename AccSel<T, KAHAN>::type acc[STREAM_MAXJ];
#pragma unroll
    for (int jj = 0; jj < STREAM_MAXJ; ++jj) acc[jj].init();
    bool failed = false;   // after an expired wait: walk on (named barriers) without work
    while (w.next(k, COL, r0, r1, item_done)) {
        const uint32_t slot = c % STREAM_NS;
        if (!failed) {
            const bool ok = mbar_wait_bounded(full + slot, (c / STREAM_NS) & 1u, &g_device_error);
            failed = __any_sync(0xffffffffu, !ok);
        }
        const unsigned char* base = ring + slot * STREAM_SLOT;
        const uint32_t mis = (uint32_t)(reinterpret_cast<uintptr_t>(A + r0 * k.L) & 15u);
        const TA* rows = reinterpret_cast<const TA*>(base + mis);
        const uint64_t s = r0 / k.nq;
        const uint64_t i0 = r0 - s * k.nq;
        const uint64_t nrows = r1 - r0;
        if (active && !failed) {
            // rows of this thread's row group: global i == rg (mod RG)
            uint64_t first = (rg + RG - (uint32_t)(i0 % RG)) % RG;
            for (uint64_t rr = first; rr < nrows; rr += RG) {
                const T bb = __ldg(Bv + i0 + rr);
                const TA* rp = rows + rr * P;
#pragma unroll
                for (int jj = 0; jj < STREAM_MAXJ; ++jj)
                    if ((uint32_t)jj < J) {
                        const uint64_t j = j0 + (uint64_t)jj * STREAM_NT;
                        if (j < P) acc[jj].fma_add(Cvt<TA, T>::f(rp[j]), bb);
                    }
            }
        }
        __syncwarp();
        if (lane == 0 && !failed) mbar_arrive(empty + slot);
        ++c;
        if (item_done) {
            // item (s, segment) complete: reduce row groups in fixed order, write
            const uint64_t item = w.unit;
            const uint64_t seg = item - s * k.nseg;
#pragma unroll
            for (int jj = 0; jj < STREAM_MAXJ; ++jj) acc[jj].fold();
            if (RG > 1) {
                T* red = sbuf;
                if (active) {
                    red[2 * ct] = acc[0].s;
                    red[2 * ct + 1] = acc[0].c;
                }
                consumer_sync();
                if (active && rg == 0) {
                    for (uint32_t g = 1; g < RG; ++g) acc[0].merge(red[2 * (g * P + j0)], red[2 * (g * P + j0) + 1]);
                }
                consumer_sync();
            }
            if (active && rg == 0 && !failed) {
#pragma unroll
                for (int jj = 0; jj < STREAM_MAXJ; ++jj)
                    if ((uint32_t)jj < J) {
                        const uint64_t j = j0 + (uint64_t)jj * STREAM_NT;
                        if (j < P) {
                            if (k.nseg == 1) {
                                static_cast<T*>(k.out)[s * P + j] = acc[jj].value();
                            } else {
                                Pair<T> pr;
                                pr.s = acc[jj].s;
                                pr.c = KAHAN ? acc[jj].c : T(0);
                                static_cast<Pair<T>*>(k.partial)[seg * (k.S * P) + s * P + j] = pr;
                            }
                        }
                    }
            }
#pragma unroll
            for (int jj = 0; jj < STREAM_MAXJ; ++jj) acc[jj].init();
        }
    }
}

}  // namespace tlibg
