// Column kernel for thin prefixes (included by ttv_kernels.cu).
//
// When P is small (P / V lanes cover a row of the prefix and P / V divides
// 32) and there are too few outputs S * P to give every lane of the plain
// column kernel an output, a warp reads RG = 32 V / P consecutive rows of a
// slab per step: lane L owns outputs j = (L mod P/V) * V .. + V - 1 of row
// group g = L / (P/V), so each warp load covers 32 V contiguous elements.
// The 8 warps of a CTA interleave along the contracted mode; a work item is
// one (segment of q, slab s).  Lanes of the same outputs are reduced by
// shuffles, the warps through shared memory in fixed order, segments by the
// deterministic combine kernel.  Every lane is busy whatever P and S are.
#pragma once

namespace tlibg {

template <typename TA, typename T, int V, bool KAHAN>
__global__ void __launch_bounds__(BLOCK, (min_ctas<TA, V>())) col_thin_kernel(KArgs k)
{
    pdl_prologue();
    constexpr int NW = BLOCK / 32;
    constexpr int U = loads_in_flight<TA, V>();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
    int* abort_flag = reinterpret_cast<int*>(smem_raw + 8);
    T* sb = reinterpret_cast<T*>(smem_raw + 16);
    constexpr int BCAP = BSTAGE_BYTES / (int)sizeof(T) + 16 / (int)sizeof(T);
    constexpr bool PRES = presplit_b<T, KAHAN>();
    float2* bsplit = reinterpret_cast<float2*>(smem_raw + 16 + BCAP * sizeof(T));
    T* red = reinterpret_cast<T*>(smem_raw + 16 + BCAP * sizeof(T) +
                                  (PRES ? BCAP * sizeof(float2) : 0));   // [NW][32][V][2]
    bool b_split_ok = false;

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t P = k.P;
    const uint32_t PV = (uint32_t)(P / V);   // lanes per row
    const uint32_t RG = 32u / PV;            // rows per warp step
    const uint32_t g = lane / PV;
    const uint64_t j0 = (uint64_t)(lane % PV) * V;
    const uint32_t step = NW * RG;           // rows between a lane's consecutive loads
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);

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
        const uint64_t s = item - seg * k.S;
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

        typename AccSel<T, KAHAN>::type acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        const TA* ap = A + s * k.nq * P + j0;
        if constexpr (PRES) {
            if (b_split_ok)
                col_loop<U, V, true>(acc, ap, P, bs, bsp, ib + warp * RG + g, ie, step);
            else
                col_loop<U, V, false>(acc, ap, P, bs, bsp, ib + warp * RG + g, ie, step);
        } else {
            col_loop<U, V, false>(acc, ap, P, bs, bsp, ib + warp * RG + g, ie, step);
        }
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].fold();
        // lanes of the same outputs (row groups g) in the warp, then the warps
        for (uint32_t o = PV; o < 32u; o <<= 1) {
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const T os = __shfl_xor_sync(0xffffffffu, acc[v].s, o);
                const T oc = __shfl_xor_sync(0xffffffffu, acc[v].c, o);
                acc[v].merge(os, oc);
            }
        }
        if (lane < PV) {
            T* r = red + ((size_t)warp * 32u + lane) * (2 * V);
#pragma unroll
            for (int v = 0; v < V; ++v) {
                r[2 * v] = acc[v].s;
                r[2 * v + 1] = acc[v].c;
            }
        }
        __syncthreads();
        if (warp == 0 && lane < PV) {
            for (uint32_t w = 1; w < (uint32_t)NW; ++w) {
                const T* r = red + ((size_t)w * 32u + lane) * (2 * V);
#pragma unroll
                for (int v = 0; v < V; ++v) acc[v].merge(r[2 * v], r[2 * v + 1]);
            }
            const uint64_t o0 = s * P + j0;
            if (k.nseg == 1) {
                T* out = static_cast<T*>(k.out) + o0;
#pragma unroll
                for (int v = 0; v < V; ++v) out[v] = acc[v].value();
            } else {
                Pair<T>* pp = static_cast<Pair<T>*>(k.partial) + seg * (k.S * P) + o0;
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    Pair<T> pr;
                    pr.s = acc[v].s;
                    pr.c = KAHAN ? acc[v].c : T(0);
                    pp[v] = pr;
                }
            }
        }
        __syncthreads();   // red is reused by the next item
    }
}

}  // namespace tlibg
