// Column kernel for scalar loads with several outputs per thread (included by
// ttv_kernels.cu).
//
// Prefixes whose rows allow no vector load (P odd, or A at an odd element
// offset): each thread owns MO outputs 32 apart (o, o + 32, ...), so every
// warp load of every output set is still one coalesced run of 32 elements,
// and each row i puts MO independent loads in flight per thread instead of
// one.  Short contractions (a few dozen rows) then need half the round trips
// per output.  Tiles, the b stage (and its double-float split for fp64),
// warps stacked along q and the split reduction are those of the column
// kernel.  Measured on GB300 ahead of the realigning kernel for every
// unaligned prefix of the sweeps, which is why that one is only on request.
#pragma once

namespace tlibg {

// Scalar loads each thread keeps in flight (over its MO outputs): 16 for
// 8-byte elements, 24 for narrower ones.  Measured on GB300 over the
// symmetric sweep's unaligned prefixes: fp32 5.37 / 5.71 / 5.69 TB/s with
// 16 / 24 / 32 loads, fp64 6.07 / 5.38 / 5.58 TB/s (fp64 carries the
// double-float state per output, so more loads cost it occupancy).
#ifndef TLIBG_STRIDED_LOADS_WIDE
#define TLIBG_STRIDED_LOADS_WIDE 16
#endif
#ifndef TLIBG_STRIDED_LOADS_NARROW
#define TLIBG_STRIDED_LOADS_NARROW 24
#endif
template <typename TA> __device__ __forceinline__ constexpr int strided_loads()
{
    return sizeof(TA) >= 8 ? TLIBG_STRIDED_LOADS_WIDE : TLIBG_STRIDED_LOADS_NARROW;
}

// 8-byte elements load through L1 with default caching: the sector a warp's
// unaligned run shares with the next run is then an L1 hit (fp64 +4 % over
// streaming loads on the symmetric sweep; fp32 the same with streaming, L1 or
// L2-only loads, so it streams).
template <typename TA> __device__ __forceinline__ constexpr bool strided_l1() { return sizeof(TA) == 8; }

// UB rows of the contracted mode: MO loads per row, all loads first.  rp[m]
// points at the thread's element of output m in the current row and moves
// on by `step` elements (WI rows) per row: one pointer add per load.
template <int UB, int MO, bool PRE, typename TA, typename T, typename AccT>
__device__ __forceinline__ void strided_rows(AccT (&acc)[MO], const TA* (&rp)[MO], uint64_t step, const T* bs,
                                             const float2* bsp, uint64_t i, uint32_t WI)
{
    T av[UB][MO];
#pragma unroll
    for (int u = 0; u < UB; ++u)
#pragma unroll
        for (int m = 0; m < MO; ++m) {
            T x[1];
            if constexpr (strided_l1<TA>())
                load_a_l1<TA, T, 1>(rp[m], x);
            else
                load_a<TA, T, 1>(rp[m], x);
            av[u][m] = x[0];
            rp[m] += step;
        }
#pragma unroll
    for (int u = 0; u < UB; ++u) row_fma<MO, PRE>(acc, av[u], bs[i + u * WI], u, PRE ? bsp + i + u * WI : nullptr);
    renorm_all<MO>(acc);
}

template <int U, int MO, bool PRE, typename TA, typename T, typename AccT>
__device__ __forceinline__ void strided_loop(AccT (&acc)[MO], const TA* (&rp)[MO], uint64_t step, const T* bs,
                                             const float2* bsp, uint64_t i, uint64_t ie, uint32_t WI)
{
    for (; i + (U - 1) * WI < ie; i += U * WI) strided_rows<U, MO, PRE>(acc, rp, step, bs, bsp, i, WI);
    if constexpr (U >= 4) {
        if (i + (U / 2 - 1) * WI < ie) {
            strided_rows<U / 2, MO, PRE>(acc, rp, step, bs, bsp, i, WI);
            i += (U / 2) * WI;
        }
    }
    if constexpr (U >= 8) {
        if (i + (U / 4 - 1) * WI < ie) {
            strided_rows<U / 4, MO, PRE>(acc, rp, step, bs, bsp, i, WI);
            i += (U / 4) * WI;
        }
    }
    for (; i < ie; i += WI) strided_rows<1, MO, PRE>(acc, rp, step, bs, bsp, i, WI);
}

template <typename TA, typename T, int MO, bool KAHAN>
__global__ void __launch_bounds__(BLOCK) col_strided_kernel(KArgs k)
{
    pdl_prologue();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    int* abort_flag = reinterpret_cast<int*>(smem_raw + 8);
    T* sb = reinterpret_cast<T*>(smem_raw + 16);
    constexpr int BCAP = BSTAGE_BYTES / (int)sizeof(T) + 16 / (int)sizeof(T);
    constexpr bool PRES = presplit_b<T, KAHAN>();
    float2* bsplit = reinterpret_cast<float2*>(smem_raw + 16 + BCAP * sizeof(T));
    T* red = reinterpret_cast<T*>(smem_raw + 16 + BCAP * sizeof(T) + (PRES ? BCAP * sizeof(float2) : 0));
    bool b_split_ok = false;

    const uint32_t WI = k.group;
    const uint32_t WO = (BLOCK / 32) / WI;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t wi = warp % WI, wo = warp / WI;
    const uint64_t TO = uint64_t(WO) * 32u * MO;
    const uint64_t P = k.P;
    const uint64_t outputs = k.S * P;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    constexpr int U = (strided_loads<TA>() / MO) < 1 ? 1 : strided_loads<TA>() / MO;

    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        *abort_flag = 0;
        fence_mbar_init();
    }
    __syncthreads();

    uint32_t phase = 0;
    uint64_t staged_seg = ~uint64_t(0);
    uint32_t off = 0;
    const uint64_t first = uint64_t(blockIdx.x) * k.items_per_cta;
    const uint64_t last = min(k.items, first + k.items_per_cta);

    for (uint64_t item = first; item < last; ++item) {
        const uint64_t seg = idx_div(item, k.tdiv);
        const uint64_t tile = item - seg * k.ntiles;
        const uint64_t ib = seg * k.seg_len;
        const uint64_t ie = min(k.nq, ib + k.seg_len);
        if (seg != staged_seg) {
            __syncthreads();   // every reader of the previous segment is done
            if (!stage_b<T>(sb, B, ib, ie, bar, phase, abort_flag, &g_device_error)) return;
            staged_seg = seg;
            off = (uint32_t)((reinterpret_cast<uintptr_t>(B + ib) & 15u) / sizeof(T));
            if constexpr (PRES) b_split_ok = stage_b_split<T>(sb + off, (uint32_t)(ie - ib), bsplit);
        }
        const T* bs = sb + off - ib;   // bs[i] = b[i] for i in [ib, ie)
        const float2* bsp = bsplit - ib;

        const uint64_t o0 = tile * TO + uint64_t(wo) * 32u * MO + lane;   // outputs o0 + 32 m
        bool ok[MO];
#pragma unroll
        for (int m = 0; m < MO; ++m) ok[m] = o0 + 32u * m < outputs;
        typename AccSel<T, KAHAN>::type acc[MO];
#pragma unroll
        for (int m = 0; m < MO; ++m) acc[m].init();
        if (ok[0]) {
            // an output past the end re-reads output o0's elements (no load
            // predicates; its sum is never stored)
            const TA* rp[MO];
            const uint64_t row0 = (ib + wi) * P;
#pragma unroll
            for (int m = 0; m < MO; ++m) {
                const uint64_t o = ok[m] ? o0 + 32u * m : o0;
                const uint64_t s = idx_div(o, k.pdiv);
                rp[m] = A + s * k.nq * P + (o - s * P) + row0;
            }
            const uint64_t step = uint64_t(WI) * P;
            if constexpr (PRES) {
                if (b_split_ok)
                    strided_loop<U, MO, true>(acc, rp, step, bs, bsp, ib + wi, ie, WI);
                else
                    strided_loop<U, MO, false>(acc, rp, step, bs, bsp, ib + wi, ie, WI);
            } else {
                strided_loop<U, MO, false>(acc, rp, step, bs, bsp, ib + wi, ie, WI);
            }
        }
#pragma unroll
        for (int m = 0; m < MO; ++m) acc[m].fold();
        if (WI > 1) {
            // warps stacked along i hand their partials to warp row wi == 0
            const uint32_t slot = wo * 32u + lane;
            if (wi > 0) {
                T* r = red + ((size_t)(wi - 1) * (WO * 32u) + slot) * (2 * MO);
#pragma unroll
                for (int m = 0; m < MO; ++m) {
                    r[2 * m] = acc[m].s;
                    r[2 * m + 1] = acc[m].c;
                }
            }
            __syncthreads();
            if (wi == 0) {
                for (uint32_t w = 1; w < WI; ++w) {
                    const T* r = red + ((size_t)(w - 1) * (WO * 32u) + slot) * (2 * MO);
#pragma unroll
                    for (int m = 0; m < MO; ++m) acc[m].merge(r[2 * m], r[2 * m + 1]);
                }
            }
            __syncthreads();
        }
        if (wi == 0) {
#pragma unroll
            for (int m = 0; m < MO; ++m) {
                if (!ok[m]) continue;
                const uint64_t o = o0 + 32u * m;
                if (k.nseg == 1) {
                    static_cast<T*>(k.out)[o] = acc[m].value();
                } else {
                    Pair<T> pr;
                    pr.s = acc[m].s;
                    pr.c = KAHAN ? acc[m].c : T(0);
                    static_cast<Pair<T>*>(k.partial)[seg * outputs + o] = pr;
                }
            }
        }
    }
}

}  // namespace tlibg
