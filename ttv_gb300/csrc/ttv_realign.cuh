// Column kernel for prefixes whose rows are not 16-byte aligned (included by
// ttv_kernels.cu).
//
// When P is not a multiple of the 16-byte vector width (V = 4 fp32, 2 fp64),
// or A starts at an odd element offset, the rows A[s, i, :] start at
// different offsets inside their 16-byte blocks and the plain column kernel
// falls back to scalar loads.  Here a warp owns a window of 32*V consecutive
// outputs of one row of one slab and, for every row i, loads the 33 aligned
// 16-byte vectors that cover the window: lane L the L-th, lane 31 also the
// 33rd when the window is misaligned.  Element v of lane L's vector belongs
// to output V L + v - r of the window, r the row's misalignment (warp-uniform,
// 0..V-1).  Instead of moving data between lanes every row, each lane keeps
// 2V - 1 accumulators, for outputs V L - (V - 1) .. V L + V - 1, and adds each
// element into the one its row's shift names (a warp-uniform switch on r, so
// every index is a compile-time constant); after the last row, one warp
// shuffle hands each lane's V - 1 low accumulators to its left neighbour,
// whose outputs they are (lane 0's belong to the previous window, whose lane
// 31 read the same elements from its 33rd vector).  Every load is a full
// 16-byte load and contains at least one element of the window, so no access
// leaves A's allocation.  Windows that
// straddle two slabs or end past a row (the last window of each row) take
// scalar loads.  Work items, the b stage, the warps stacked along q and the
// split reduction are those of the column kernel.  Chosen only on request
// (TLIBG_KIND_COL_REALIGN): the strided kernel's scalar loads with two
// outputs per thread measured faster on every unaligned prefix of the sweeps.
#pragma once

namespace tlibg {

// w[BASE + v] += av[v] * bb for v < NV (the fp64 mix alternates native and
// emulated products over (u, v) as row_fma does).
template <int V, bool PRE, int BASE, int NV, typename AccT, typename T>
__device__ __forceinline__ void win_fma(AccT* w, const T (&av)[V], T bb, int u, const float2* bsp)
{
    if constexpr (std::is_same<AccT, AccDF>::value) {
        DSplit bs;
        if constexpr (PRE) {
            const float2 t = *bsp;
            bs.hi = t.x;
            bs.lo = t.y;
            bs.ok = true;
        } else {
            bs = split_double(bb);
        }
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            if (f64_native<V>(u, v))
                w[BASE + v].d = fma(av[v], bb, w[BASE + v].d);
            else
                w[BASE + v].add_split(split_double(av[v]), bs, av[v], bb);
        }
    } else {
#pragma unroll
        for (int v = 0; v < NV; ++v) w[BASE + v].fma_add(av[v], bb);
    }
}

// One row of a lane: its vector (shift r) and, for lane 31, the 33rd vector.
template <int V, bool PRE, typename AccT, typename T>
__device__ __forceinline__ void win_row(AccT* w, const T (&cur)[V], const T (&ext)[V], uint32_t r, bool last,
                                        T bb, int u, const float2* bsp)
{
    switch (r) {
    case 0:
        win_fma<V, PRE, V - 1, V>(w, cur, bb, u, bsp);
        break;
    case 1:
        win_fma<V, PRE, V - 2, V>(w, cur, bb, u, bsp);
        if (last) win_fma<V, PRE, 2 * V - 2, 1>(w, ext, bb, u, bsp);
        break;
    case 2:
        if constexpr (V > 2) {
            win_fma<V, PRE, V - 3, V>(w, cur, bb, u, bsp);
            if (last) win_fma<V, PRE, 2 * V - 3, 2>(w, ext, bb, u, bsp);
        }
        break;
    default:
        if constexpr (V > 3) {
            win_fma<V, PRE, V - 4, V>(w, cur, bb, u, bsp);
            if (last) win_fma<V, PRE, 2 * V - 4, 3>(w, ext, bb, u, bsp);
        }
        break;
    }
}

// After the last row: lane L's accumulators 0..V-2 are outputs of lane L - 1;
// acc[v] = w[V - 1 + v] plus the right neighbour's w[v - 1] (none for lane 31).
template <int V, typename T, bool KAHAN>
__device__ __forceinline__ void win_collect(Acc<T, KAHAN> (&w)[2 * V - 1], Acc<T, KAHAN> (&acc)[V], uint32_t lane)
{
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = w[V - 1 + v];
#pragma unroll
    for (int v = 1; v < V; ++v) {
        const T os = __shfl_down_sync(0xffffffffu, w[v - 1].s, 1);
        const T oc = __shfl_down_sync(0xffffffffu, w[v - 1].c, 1);
        if (lane < 31u) acc[v].merge(os, oc);
    }
}
template <int V>
__device__ __forceinline__ void win_collect(AccDF (&w)[2 * V - 1], AccDF (&acc)[V], uint32_t lane)
{
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v] = w[V - 1 + v];
#pragma unroll
    for (int v = 1; v < V; ++v) {
        AccDF o;
        o.hi = __shfl_down_sync(0xffffffffu, w[v - 1].hi, 1);
        o.lo = __shfl_down_sync(0xffffffffu, w[v - 1].lo, 1);
        o.d = __shfl_down_sync(0xffffffffu, w[v - 1].d, 1);
        if (lane < 31u) acc[v].absorb(o);
    }
}

template <typename T, bool KAHAN>
__global__ void __launch_bounds__(BLOCK) col_realign_kernel(KArgs k)
{
    pdl_prologue();
    constexpr int V = 16 / (int)sizeof(T);
    constexpr int U = 4;
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
    const uint64_t TO = uint64_t(WO) * 32u * V;
    const uint64_t P = k.P;
    const uint64_t outputs = k.S * P;
    const T* __restrict__ A = static_cast<const T*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    // A's element offset inside its 16-byte block
    const uint32_t amis = (uint32_t)((reinterpret_cast<uintptr_t>(A) & 15u) / sizeof(T));

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

        const uint64_t ow = tile * TO + uint64_t(wo) * 32u * V;   // the warp's window
        const uint64_t o0 = ow + uint64_t(lane) * V;
        typename AccSel<T, KAHAN>::type acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        if (ow < outputs) {
            const uint64_t sw = idx_div(ow, k.pdiv);
            const uint64_t jw = ow - sw * P;
            if (jw + 32u * V <= P) {
                // whole window inside row (sw, i, .): aligned vector loads, shifted accumulators
                const uint64_t base = sw * k.nq * P + jw;   // element index of A[sw, 0, jw]
                typename AccSel<T, KAHAN>::type w[2 * V - 1];
#pragma unroll
                for (int v = 0; v < 2 * V - 1; ++v) w[v].init();
                const bool last_lane = lane == 31u;
                const bool pre = PRES && b_split_ok;
                uint64_t i = ib + wi;
                for (; i + (U - 1) * WI < ie; i += U * WI) {
                    T cur[U][V], ext[U][V] = {};
                    uint32_t r[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const uint64_t e = base + (i + u * WI) * P;
                        r[u] = (uint32_t)((amis + e) & (V - 1));
                        const T* vp = A + (int64_t)(e - r[u]);   // 16-byte aligned, in A's first block at worst
                        load_a<T, T, V>(vp + lane * V, cur[u]);
                        if (last_lane && r[u] != 0u) load_a<T, T, V>(vp + 32u * V, ext[u]);
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (pre)
                            win_row<V, PRES>(w, cur[u], ext[u], r[u], last_lane, bs[i + u * WI], u,
                                             bsp + i + u * WI);
                        else
                            win_row<V, false>(w, cur[u], ext[u], r[u], last_lane, bs[i + u * WI], u, nullptr);
                    }
                    renorm_all<2 * V - 1>(w);
                }
                for (; i < ie; i += WI) {
                    T cur[V], ext[V] = {};
                    const uint64_t e = base + i * P;
                    const uint32_t rr = (uint32_t)((amis + e) & (V - 1));
                    const T* vp = A + (int64_t)(e - rr);
                    load_a<T, T, V>(vp + lane * V, cur);
                    if (last_lane && rr != 0u) load_a<T, T, V>(vp + 32u * V, ext);
                    if (pre)
                        win_row<V, PRES>(w, cur, ext, rr, last_lane, bs[i], 0, bsp + i);
                    else
                        win_row<V, false>(w, cur, ext, rr, last_lane, bs[i], 0, nullptr);
                    renorm_all<2 * V - 1>(w);
                }
                win_collect<V>(w, acc, lane);
            } else {
                // window straddles two slabs or ends past the row: scalar loads
                uint64_t ofs[V];
                bool ok[V];
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const uint64_t o = o0 + v;
                    ok[v] = o < outputs;
                    const uint64_t s = ok[v] ? idx_div(o, k.pdiv) : 0;
                    ofs[v] = s * k.nq * P + (o - s * P);
                }
                for (uint64_t i = ib + wi; i < ie; i += WI) {
                    const T bb = bs[i];
#pragma unroll
                    for (int v = 0; v < V; ++v)
                        if (ok[v]) {
                            T av[1];
                            load_a<T, T, 1>(A + ofs[v] + i * P, av);
                            acc[v].fma_add(av[0], bb);
                        }
                }
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].fold();
        if (WI > 1) {
            // warps stacked along i hand their partials to warp row wi == 0
            const uint32_t slot = wo * 32u + lane;
            if (wi > 0) {
                T* rp = red + ((size_t)(wi - 1) * (WO * 32u) + slot) * (2 * V);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    rp[2 * v] = acc[v].s;
                    rp[2 * v + 1] = acc[v].c;
                }
            }
            __syncthreads();
            if (wi == 0) {
                for (uint32_t w = 1; w < WI; ++w) {
                    const T* rp = red + ((size_t)(w - 1) * (WO * 32u) + slot) * (2 * V);
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v].merge(rp[2 * v], rp[2 * v + 1]);
                }
            }
            __syncthreads();
        }
        if (wi == 0) {
            if (k.nseg == 1) {
                T* out = static_cast<T*>(k.out) + o0;
                if (o0 + V <= outputs && (reinterpret_cast<uintptr_t>(out) & 15u) == 0) {
                    T vals[V];
#pragma unroll
                    for (int v = 0; v < V; ++v) vals[v] = acc[v].value();
                    *reinterpret_cast<uint4*>(out) = *reinterpret_cast<const uint4*>(vals);
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v)
                        if (o0 + v < outputs) out[v] = acc[v].value();
                }
            } else {
                Pair<T>* pp = static_cast<Pair<T>*>(k.partial) + seg * outputs;
#pragma unroll
                for (int v = 0; v < V; ++v)
                    if (o0 + v < outputs) {
                        Pair<T> pr;
                        pr.s = acc[v].s;
                        pr.c = KAHAN ? acc[v].c : T(0);
                        pp[o0 + v] = pr;
                    }
            }
        }
    }
}

}  // namespace tlibg
