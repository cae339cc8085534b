// Shared by the row-tile and streamed kernels (ttv_kernels.cu) and the
// batched executor's row-tile units (ttv_batch.cu): the 1-D TMA bulk copy of
// a contiguous run of A into a shared-memory stage (ragged head and tail by
// plain loads), and the one-lane-per-row walk over rows held in shared memory.
#pragma once

#include <type_traits>

#include "ttv_device.cuh"

namespace tlibg {

// Copy A[e0, e1) into `slot` so that element e lands at byte
//   (A + e) - ((A + e0) & ~15)
// of the slot: the 16-byte-aligned body with one cp.async.bulk issued by lane
// 0 against `full` (expect_tx), the ragged head and tail (under 16 bytes
// each) by lanes 0-15 and 16-31 with plain loads.  Called by a whole warp.
template <typename TA>
__device__ __forceinline__ void stream_issue(const TA* A, uint64_t e0, uint64_t e1, unsigned char* slot,
                                             uint64_t* full, uint32_t lane)
{
    const uintptr_t g0 = reinterpret_cast<uintptr_t>(A + e0);
    const uintptr_t g1 = reinterpret_cast<uintptr_t>(A + e1);
    const uintptr_t base = g0 & ~uintptr_t(15);
    uintptr_t body0 = (g0 + 15) & ~uintptr_t(15);
    uintptr_t body1 = g1 & ~uintptr_t(15);
    if (body0 > g1) body0 = g1;
    if (body1 < body0) body1 = body0;
    // ragged head [g0, body0) and tail [body1, g1): element-wise plain loads
    const uint32_t head = (uint32_t)((body0 - g0) / sizeof(TA));
    const uint32_t tail = (uint32_t)((g1 - body1) / sizeof(TA));
    if (lane < head) {
        const TA* src = reinterpret_cast<const TA*>(g0) + lane;
        *reinterpret_cast<TA*>(slot + (reinterpret_cast<uintptr_t>(src) - base)) = *src;
    } else if (lane >= 16 && lane - 16 < tail) {
        const TA* src = reinterpret_cast<const TA*>(body1) + (lane - 16);
        *reinterpret_cast<TA*>(slot + (reinterpret_cast<uintptr_t>(src) - base)) = *src;
    }
    __syncwarp();
    if (lane == 0) {
        const uint32_t bytes = (uint32_t)(body1 - body0);
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(full, bytes);
        if (bytes) bulk_g2s(slot + (body0 - base), reinterpret_cast<const void*>(body0), bytes, full);
    }
}


#ifndef TLIBG_ROWT_NATIVE_EVERY
#define TLIBG_ROWT_NATIVE_EVERY 2
#endif

// One step of R rows at column c: element c of each row times b[c].
template <int R, bool NATIVE, bool PRE, typename TA, typename T, typename AccT>
__device__ __forceinline__ void rowt_step(AccT (&acc)[R], const TA* (&rp)[R], const T* sb, const float2* bsp,
                                          uint32_t c)
{
    const T bb = sb[c];
    if constexpr (std::is_same<AccT, AccDF>::value) {
        if constexpr (NATIVE) {
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r].d = fma((double)rp[r][c], bb, acc[r].d);
        } else {
            DSplit bs;
            if constexpr (PRE) {
                const float2 t = bsp[c];
                bs.hi = t.x;
                bs.lo = t.y;
                bs.ok = true;
            } else {
                bs = split_double(bb);
            }
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const double a = rp[r][c];
                acc[r].add_split(split_double(a), bs, a, bb);
            }
        }
    } else {
#pragma unroll
        for (int r = 0; r < R; ++r) acc[r].fma_add(Cvt<TA, T>::f(rp[r][c]), bb);
    }
}

// Next column of the walk: wrapping at n_q (rotated walks of even n_q), or
// straight (odd n_q, which starts at column 0).
template <bool WRAP> __device__ __forceinline__ uint32_t rowt_next(uint32_t c, uint32_t nq)
{
    if constexpr (WRAP) return (c + 1 == nq) ? 0u : c + 1;
    return c + 1;
}

// The lane's R rows (rp[r]) over all n_q columns, walking from column c.
// fp64 with the double-float mix: the first step of every
// TLIBG_ROWT_NATIVE_EVERY on the DFMA pipe, the rest emulated, in blocks of
// RT_G such groups with one renormalisation each (at most 8 emulated
// products between two); the last n_q mod E steps native.
constexpr int RT_G = 4;
template <int R, bool PRE, bool WRAP, typename TA, typename T, typename AccT>
__device__ __forceinline__ void rowt_dot(AccT (&acc)[R], const TA* (&rp)[R], const T* sb, const float2* bsp,
                                         uint32_t nq, uint32_t c)
{
    if constexpr (std::is_same<AccT, AccDF>::value) {
        constexpr int E = TLIBG_ROWT_NATIVE_EVERY;
        static_assert(RT_G * (E - 1) <= 8, "renormalise at least every 8 emulated products");
        uint32_t j = 0;
        for (; j + RT_G * E <= nq; j += RT_G * E) {
#pragma unroll
            for (int gq = 0; gq < RT_G; ++gq) {
                rowt_step<R, true, PRE>(acc, rp, sb, bsp, c);
                c = rowt_next<WRAP>(c, nq);
#pragma unroll
                for (int u = 1; u < E; ++u) {
                    rowt_step<R, false, PRE>(acc, rp, sb, bsp, c);
                    c = rowt_next<WRAP>(c, nq);
                }
            }
#pragma unroll
            for (int r = 0; r < R; ++r) acc[r].renorm();
        }
        for (; j + E <= nq; j += E) {   // fewer than RT_G groups left: fold() renormalises
            rowt_step<R, true, PRE>(acc, rp, sb, bsp, c);
            c = rowt_next<WRAP>(c, nq);
#pragma unroll
            for (int u = 1; u < E; ++u) {
                rowt_step<R, false, PRE>(acc, rp, sb, bsp, c);
                c = rowt_next<WRAP>(c, nq);
            }
        }
        for (; j < nq; ++j) {
            rowt_step<R, true, PRE>(acc, rp, sb, bsp, c);
            c = rowt_next<WRAP>(c, nq);
        }
    } else {
        uint32_t j = 0;
        for (; j + 8 <= nq; j += 8) {
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                rowt_step<R, true, PRE>(acc, rp, sb, bsp, c);
                c = rowt_next<WRAP>(c, nq);
            }
        }
        for (; j < nq; ++j) {
            rowt_step<R, true, PRE>(acc, rp, sb, bsp, c);
            c = rowt_next<WRAP>(c, nq);
        }
    }
}

// Even n_q walks rotated (wrapping), odd n_q straight.
template <int R, bool PRE, typename TA, typename T, typename AccT>
__device__ __forceinline__ void rowt_dot_any(AccT (&acc)[R], const TA* (&rp)[R], const T* sb, const float2* bsp,
                                             uint32_t nq, uint32_t c)
{
    if (nq & 1u)
        rowt_dot<R, PRE, false>(acc, rp, sb, bsp, nq, 0u);
    else
        rowt_dot<R, PRE, true>(acc, rp, sb, bsp, nq, c);
}

}  // namespace tlibg
