// Row-tile kernel for short q-fastest rows (included by ttv_kernels.cu,
// after ttv_stream.cuh, whose bulk-copy issue it shares).
//
// P == 1, n_q <= ROWT_MAX_NQ, no split.  One lane owns R rows (R = 1, 2 or 4,
// so that a tile holds about 4 KB of A), so a row needs no cross-lane
// reduction, and a warp owns tiles of 32 R consecutive rows: one contiguous
// run of A.  Each warp moves its tiles into its own ring of
// ROWT_NS shared-memory stages with one 1-D TMA bulk copy per tile (the
// ragged head and tail, under 16 bytes each, by plain loads, so any alignment
// works), waits on the stage's mbarrier (bounded) and then reads its rows
// from shared memory.  Every HBM access stays coalesced: a lane reading its
// own row straight from global memory touches 32 lines per warp load, which
// saturated L1 on rows of 16 doubles.  With n_q even the lanes start their
// walk along the row at a lane-dependent column (wrapping around), so the
// lanes of one shared-memory read hit distinct banks; odd n_q strides apart
// already.  b, and for fp64 its double-float split, sit in shared memory.
// fp64 mixes native DFMA with the double-float emulation (one product in
// TLIBG_ROWT_NATIVE_EVERY native), fp32 / bf16 use the Kahan accumulator.
#pragma once

#include "ttv_rowwalk.cuh"

namespace tlibg {


// Shared memory of the kernel: mbarriers (128 bytes), b, b's split (fp64
// with the double-float mix), then ROWT_WARPS * ROWT_NS stages.
__host__ __device__ inline size_t rowt_b_bytes(uint64_t nq, size_t et) { return (size_t)((nq * et + 15) & ~uint64_t(15)); }
__host__ __device__ inline size_t rowt_split_bytes(uint64_t nq, bool pres) { return pres ? (size_t)((nq * 8 + 15) & ~uint64_t(15)) : 0; }

// Tile t of the warp's walk: rows [32 R t, min(S, 32 R t + 32 R)) into `slot`.
template <typename TA>
__device__ __forceinline__ void rowt_issue(const TA* A, uint64_t S, uint64_t nq, uint64_t t, uint32_t R,
                                           unsigned char* slot, uint64_t* full, uint32_t lane)
{
    const uint64_t r0 = t * 32 * R;
    const uint64_t r1 = min(S, r0 + 32 * R);
    stream_issue<TA>(A, r0 * nq, r1 * nq, slot, full, lane);
}

template <typename TA, typename T, bool KAHAN, int R>
__global__ void __launch_bounds__(ROWT_THREADS) row_tile_kernel(KArgs k)
{
    pdl_prologue();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t nq = (uint32_t)k.nq;
    constexpr bool PRES = presplit_b<T, KAHAN>();
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw) + warp * ROWT_NS;
    T* sb = reinterpret_cast<T*>(smem_raw + 128);
    const size_t b_bytes = rowt_b_bytes(nq, sizeof(T));
    float2* bsp = reinterpret_cast<float2*>(smem_raw + 128 + b_bytes);
    const size_t slot = rowt_slot_bytes(nq, sizeof(TA), R);
    unsigned char* ring = smem_raw + 128 + b_bytes + rowt_split_bytes(nq, PRES) + (size_t)warp * ROWT_NS * slot;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);

    if (lane == 0) {
        for (int s = 0; s < ROWT_NS; ++s) mbar_init(full + s, 1);
        fence_mbar_init();
    }
    for (uint32_t e = threadIdx.x; e < nq; e += ROWT_THREADS) sb[e] = __ldg(B + e);
    __syncthreads();
    bool split_ok = false;
    if constexpr (PRES) split_ok = stage_b_split<T>(sb, nq, bsp);

    const uint64_t tiles = (k.S + 32 * R - 1) / (32 * R);
    const uint64_t gw = (uint64_t)blockIdx.x * ROWT_WARPS + warp;
    const uint64_t nw = (uint64_t)gridDim.x * ROWT_WARPS;
    for (int s = 0; s < ROWT_NS; ++s) {
        const uint64_t t = gw + (uint64_t)s * nw;
        if (t < tiles) rowt_issue<TA>(A, k.S, k.nq, t, R, ring + (size_t)s * slot, full + s, lane);
    }
    // even n_q: start at a lane-dependent column so a shared-memory read by the
    // warp spreads over the banks
    const uint32_t rot = (nq & 1u) ? 0u : lane % nq;
    uint32_t c = 0;
    for (uint64_t t = gw; t < tiles; t += nw, ++c) {
        const uint32_t s = c % ROWT_NS;
        const bool ok = mbar_wait_bounded(full + s, (c / ROWT_NS) & 1u, &g_device_error);
        if (__any_sync(0xffffffffu, !ok)) {
            // leave only after this warp's copies in flight have landed (bounded)
            for (uint32_t o = 0; o < (uint32_t)ROWT_NS; ++o)
                if (t + (uint64_t)o * nw < tiles)
                    mbar_wait_bounded(full + (c + o) % ROWT_NS, ((c + o) / ROWT_NS) & 1u, &g_device_error);
            return;
        }
        const uint64_t r0 = t * 32 * R;
        const uint32_t mis = (uint32_t)(reinterpret_cast<uintptr_t>(A + r0 * k.nq) & 15u);
        const TA* rows = reinterpret_cast<const TA*>(ring + (size_t)s * slot + mis);
        typename AccSel<T, KAHAN>::type acc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r].init();
        if (r0 + lane < k.S) {
            // rows lane + 32 r of the tile; one past the end re-reads row `lane`
            // (its sum is not stored)
            const TA* rp[R];
#pragma unroll
            for (int r = 0; r < R; ++r)
                rp[r] = rows + (size_t)((r0 + lane + 32u * r < k.S) ? lane + 32u * r : lane) * nq;
            if constexpr (PRES) {
                if (split_ok)
                    rowt_dot_any<R, true>(acc, rp, sb, bsp, nq, rot);
                else
                    rowt_dot_any<R, false>(acc, rp, sb, bsp, nq, rot);
            } else {
                rowt_dot_any<R, false>(acc, rp, sb, bsp, nq, rot);
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r].fold();
        __syncwarp();   // every lane is done with the stage
        const uint64_t tn = t + (uint64_t)ROWT_NS * nw;
        if (tn < tiles) rowt_issue<TA>(A, k.S, k.nq, tn, R, ring + (size_t)s * slot, full + s, lane);
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint64_t row = r0 + lane + 32u * r;
            if (row < k.S) static_cast<T*>(k.out)[row] = acc[r].value();
        }
    }
}

}  // namespace tlibg
