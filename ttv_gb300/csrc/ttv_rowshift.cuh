// Row kernel for rows that are not whole 16-byte vectors (included by
// ttv_kernels.cu).
//
// P == 1 with n_q not a multiple of V = 16 / sizeof(T) (rows of 645 or 625
// floats): consecutive rows start at every misalignment m in [0, V), so the
// plain row kernel falls back to scalar loads.  Here every row is read as its
// 16-byte-aligned body (vector loads) plus at most V - 1 head and V - 1 tail
// elements (scalar loads); no load leaves the row.  The body's first vector
// holds row element (V - m) % V, so the b values that meet a body vector
// are b shifted by m: the CTA keeps V shifted copies of b in shared memory,
//   bsh[s][x] = b[x - s]   (0 outside [0, n_q)),   x in [0, W), W = n_q + V
// rounded up to V, so body vector k of a row with misalignment m meets the
// aligned vector bsh[m][x0 + kV..] with x0 = 0 (m == 0) or V.  fp64 with the
// double-float mix keeps the copies' splits beside them.
//
//   items        rows, G lanes each (the row kernel's lane rule), no split
//   per lane     body vectors gl, gl + G, ... with U loads in flight; head and
//                tail elements gl < count
//   output       the G lanes' sums meet in a warp shuffle tree (fixed order)
//
// Shared memory: V W elements of b (+ V W float2 for the fp64 mix), at most
// RS_SMEM_MAX bytes; longer rows keep the row kernel's scalar path.
#pragma once

namespace tlibg {

template <typename T, bool KAHAN>
__global__ void __launch_bounds__(BLOCK, 4) row_shift_kernel(KArgs k)
{
    pdl_prologue();
    constexpr int V = 16 / (int)sizeof(T);
    constexpr int U = 4;
    constexpr bool PRES = presplit_b<T, KAHAN>();
    typedef typename AccSel<T, KAHAN>::type AccT;
    typedef typename RawVec<16>::type R;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    const uint64_t nq = k.nq;
    const uint32_t W = (uint32_t)rs_width(nq, V);
    T* bsh = reinterpret_cast<T*>(smem_raw);
    float2* bsp = reinterpret_cast<float2*>(smem_raw + (size_t)V * W * sizeof(T));
    const T* __restrict__ B = static_cast<const T*>(k.b);
    const T* __restrict__ A = static_cast<const T*>(k.a);

    int ok = 1;
    for (uint32_t idx = threadIdx.x; idx < (uint32_t)V * W; idx += BLOCK) {
        const uint32_t s = idx / W, x = idx - s * W;
        const T v = (x >= s && x - s < nq) ? __ldg(B + (x - s)) : T(0);
        bsh[idx] = v;
        if constexpr (PRES) {
            const DSplit d = split_double((double)v);
            bsp[idx] = make_float2(d.hi, d.lo);
            ok &= (d.ok || v == T(0)) ? 1 : 0;
        }
    }
    // the emulated products need every b element inside the split's window
    bool pre_ok = false;
    if constexpr (PRES)
        pre_ok = __syncthreads_and(ok) != 0;
    else
        __syncthreads();

    const uint32_t G = k.group;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gl = lane & (G - 1u);
    const uint32_t gpw = 32u / G;
    const uint64_t warp_id = (uint64_t(blockIdx.x) * BLOCK + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * BLOCK) >> 5;
    const uintptr_t abase = reinterpret_cast<uintptr_t>(A) / sizeof(T);   // element address of A

    for (uint64_t wbase = warp_id * gpw; wbase < k.items; wbase += nwarps * gpw) {
        const uint64_t row = wbase + lane / G;
        AccT acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        if (row < k.items) {
            const uint64_t rs = row * nq;
            const uint32_t m = (uint32_t)((abase + rs) & (uint64_t)(V - 1));
            const uint64_t head = min((uint64_t)((V - m) & (V - 1)), nq);
            const uint64_t nvb = (nq - head) / V;            // body vectors
            const uint64_t tail0 = head + nvb * V;           // first tail element (row position)
            const T* ab = A + rs + head;                     // 16-byte aligned
            const uint32_t x0 = m == 0 ? 0u : (uint32_t)V;
            const T* bb = bsh + (size_t)m * W + x0;
            const float2* bp = bsp + (size_t)m * W + x0;
            uint64_t kv = gl;
            for (; kv + (U - 1) * G < nvb; kv += U * G) {
                T av[U][V], bv[U][V];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    load_a<T, T, V>(ab + (kv + u * G) * V, av[u]);
                    const R r = *reinterpret_cast<const R*>(bb + (kv + u * G) * V);
                    memcpy(bv[u], &r, 16);
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if constexpr (PRES) {
                        if (pre_ok)
                            vec_fma<V, true>(acc, av[u], bv[u], u, bp + (kv + u * G) * V);
                        else
                            vec_fma<V, false>(acc, av[u], bv[u], u);
                    } else {
                        vec_fma<V, false>(acc, av[u], bv[u], u);
                    }
                }
                renorm_all<V>(acc);
            }
            for (; kv < nvb; kv += G) {
                T av[1][V], bv[1][V];
                load_a<T, T, V>(ab + kv * V, av[0]);
                const R r = *reinterpret_cast<const R*>(bb + kv * V);
                memcpy(bv[0], &r, 16);
                if constexpr (PRES) {
                    if (pre_ok)
                        vec_fma<V, true>(acc, av[0], bv[0], 0, bp + kv * V);
                    else
                        vec_fma<V, false>(acc, av[0], bv[0], 0);
                } else {
                    vec_fma<V, false>(acc, av[0], bv[0], 0);
                }
            }
            renorm_all<V>(acc);
            // head [0, head) and tail [tail0, nq): b in place (copy 0)
            const uint64_t nt = nq - tail0;
            for (uint64_t t = gl; t < head + nt; t += G) {
                const uint64_t e = t < head ? t : tail0 + (t - head);
                T av[1];
                load_a<T, T, 1>(A + rs + e, av);
                acc[0].fma_add(av[0], bsh[e]);
            }
        }
        fold_vec<V>(acc);
        for (uint32_t off = G >> 1; off > 0; off >>= 1) {
            const T os = __shfl_xor_sync(0xffffffffu, acc[0].s, off);
            const T oc = __shfl_xor_sync(0xffffffffu, acc[0].c, off);
            acc[0].merge(os, oc);
        }
        if (row < k.items && gl == 0) static_cast<T*>(k.out)[row] = acc[0].value();
    }
}

}  // namespace tlibg
