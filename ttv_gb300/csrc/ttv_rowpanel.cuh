// Row-panel kernel: long q-fastest rows, few of them (included by
// ttv_kernels.cu).
//
// P == 1 with n_q long and S small: the asymmetric sweep's 4-256 rows of
// 2^20-2^26 elements, where b is as long as a row (up to 256 MB) and does not
// stay in L2 while A streams past it.  The row kernel's (row, segment) items
// read b again for every row segment: through L2 at best, from HBM once b no
// longer fits.  Here a work item is (segment, block of rows): the CTA loads
// its segment of b into registers once (each thread RP_K vectors, coalesced
// over the CTA), then streams that segment of every row of the block,
// reusing the registers, so b crosses the memory system once per row block
// instead of once per row.
//
//   segment      RP_K * BLOCK vectors of V elements (16 KB of b for fp32 /
//                fp64, 32 KB for bf16-stored A with fp32 b)
//   row block    `rows_per_item` consecutive rows (all S when the segments
//                alone fill the grid)
//   per row      each thread's RP_K vector loads (evict-first), RR rows in
//                flight; the lanes' partial sums meet in a warp shuffle
//                reduction, the warps' in shared memory in fixed order
//   output       one (segment, row) partial pair; combine_kernel sums the
//                segments of each row in fixed order (deterministic)
//
// Rows must allow 16-byte loads (n_q a multiple of V, A and b 16-byte
// aligned).  On request (TLIBG_KIND_ROW_PANEL) and as an autotuner candidate:
// measured on GB300 the row kernel's segment-major walk (the S rows of one b
// segment taken up by neighbouring warps, so b comes from HBM about once) is
// as fast or faster on the asymmetric sweep's rows, so the planner keeps it.
#pragma once

namespace tlibg {

constexpr int RP_RB = 8;    // rows whose warp partials are gathered per CTA barrier

template <typename TA, typename T, int V, bool KAHAN, int RR>
__global__ void __launch_bounds__(BLOCK, (min_ctas<TA, V>())) row_panel_kernel(KArgs k)
{
    pdl_prologue();
    __shared__ double s_red[BLOCK / 32][RP_RB][2];
    typedef typename AccSel<T, KAHAN>::type AccT;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint64_t L = k.seg_len;          // elements per segment (RP_K * BLOCK * V)
    const uint64_t nrb = k.ntiles;         // row blocks
    const uint64_t RBK = k.items_per_cta;  // rows per row block
    constexpr bool PRES = presplit_b<T, KAHAN>();

    for (uint64_t item = blockIdx.x; item < k.items; item += gridDim.x) {
        const uint64_t seg = item / nrb;
        const uint64_t rb = item - seg * nrb;
        const uint64_t r0 = rb * RBK;
        const uint64_t r1 = min(k.S, r0 + RBK);
        // this thread's vectors of the segment: b in registers, once per item
        T bv[RP_K][V];
        float2 bsp[RP_K][V];
        uint64_t e0[RP_K];
        bool in[RP_K];
#pragma unroll
        for (int t = 0; t < RP_K; ++t) {
            e0[t] = seg * L + ((uint64_t)t * BLOCK + threadIdx.x) * V;
            in[t] = e0[t] < k.nq;
            if (in[t]) {
                load_b<T, V>(B + e0[t], bv[t]);
            } else {
#pragma unroll
                for (int v = 0; v < V; ++v) bv[t][v] = T(0);
            }
            if constexpr (PRES) {
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    const DSplit d = split_double((double)bv[t][v]);
                    bsp[t][v] = make_float2(d.hi, d.lo);
                }
            }
        }
        // the emulated products need every b element inside the split's window
        bool pre_ok = true;
        if constexpr (PRES) {
#pragma unroll
            for (int t = 0; t < RP_K; ++t)
#pragma unroll
                for (int v = 0; v < V; ++v) pre_ok = pre_ok && split_double((double)bv[t][v]).ok;
            pre_ok = __syncthreads_and(pre_ok ? 1 : 0) != 0;
        }
        for (uint64_t rbase = r0; rbase < r1; rbase += RP_RB) {
            const uint32_t nr = (uint32_t)min((uint64_t)RP_RB, r1 - rbase);
            for (uint32_t j = 0; j < nr; j += RR) {
                T av[RR][RP_K][V];
                // all loads of RR rows first
#pragma unroll
                for (int r = 0; r < RR; ++r) {
                    const bool rok = j + r < nr;
                    const TA* ap = A + (rbase + j + r) * k.nq;
#pragma unroll
                    for (int t = 0; t < RP_K; ++t) {
                        if (rok && in[t]) {
                            load_a<TA, T, V>(ap + e0[t], av[r][t]);
                        } else {
#pragma unroll
                            for (int v = 0; v < V; ++v) av[r][t][v] = T(0);
                        }
                    }
                }
#pragma unroll
                for (int r = 0; r < RR; ++r) {
                    AccT acc[V];
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v].init();
#pragma unroll
                    for (int t = 0; t < RP_K; ++t) {
                        if constexpr (PRES) {
                            if (pre_ok)
                                vec_fma<V, true>(acc, av[r][t], bv[t], t, bsp[t]);
                            else
                                vec_fma<V, false>(acc, av[r][t], bv[t], t);
                        } else {
                            vec_fma<V, false>(acc, av[r][t], bv[t], t);
                        }
                    }
                    renorm_all<V>(acc);
                    fold_vec<V>(acc);
                    for (uint32_t off = 16; off > 0; off >>= 1) {
                        const T os = __shfl_xor_sync(0xffffffffu, acc[0].s, off);
                        const T oc = __shfl_xor_sync(0xffffffffu, acc[0].c, off);
                        acc[0].merge(os, oc);
                    }
                    if (lane == 0 && j + r < nr) {
                        s_red[warp][j + r][0] = (double)acc[0].s;
                        s_red[warp][j + r][1] = KAHAN ? (double)acc[0].c : 0.0;
                    }
                }
            }
            __syncthreads();
            if (threadIdx.x < nr) {
                // the CTA's warps in fixed order: one partial per (segment, row)
                AccT acc;
                acc.init();
                acc.s = (T)s_red[0][threadIdx.x][0];
                acc.c = (T)s_red[0][threadIdx.x][1];
                for (uint32_t w = 1; w < BLOCK / 32; ++w)
                    acc.merge((T)s_red[w][threadIdx.x][0], (T)s_red[w][threadIdx.x][1]);
                Pair<T> pr;
                pr.s = acc.s;
                pr.c = KAHAN ? acc.c : T(0);
                static_cast<Pair<T>*>(k.partial)[seg * k.S + rbase + threadIdx.x] = pr;
            }
            __syncthreads();
        }
    }
}

}  // namespace tlibg
