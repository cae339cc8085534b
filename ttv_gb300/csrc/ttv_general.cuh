// General-stride TTV (included by ttv_api.cu): tlibg_ttv_strided, an extension
// beside the drop-in calls with the natural meaning of every stride -- A's
// element (i_1..i_p) at a[sum_r i_r wa[r]], b's element i at b[i wb], C's
// element (j_1..j_{p-1}) at c[sum_r j_r wc[r]] -- for views (sliced, padded,
// transposed) that the dense kernels do not take.
//
// The outputs are numbered in a mixed radix over the modes other than q,
// sorted by A stride (fastest first), so consecutive outputs sit next to each
// other in A where the views allow it.
//   column form (q is not A's fastest mode): one output per thread; the
//     threads of a warp read neighbouring elements of each of the n_q rows,
//     eight rows in flight per thread;
//   row form (q is A's fastest mode): a group of G lanes per output (G from
//     n_q: about 16 elements per lane, 1..32), the lanes stride over the n_q
//     elements (one coalesced run per load when wa[q] == 1), a shuffle tree
//     sums the group's lanes in fixed order.
// Where the view puts rows or outputs on the 16-byte grid, the same two forms
// with 16-byte loads.  Compensated accumulation (Kahan) in the element type.
#pragma once

namespace tlibg {

constexpr int GS_MAX_MODES = 16;   // modes other than q

struct GSArgs {
    const void* a;
    const void* b;
    void* c;
    uint64_t ext[GS_MAX_MODES];   // extents of the modes other than q, A-stride order
    uint64_t wa[GS_MAX_MODES];
    uint64_t wc[GS_MAX_MODES];
    int nm;
    uint64_t outputs;             // product of ext
    uint64_t nq, waq, wb;
    uint32_t group;               // row form: lanes per output
};

__device__ __forceinline__ void gs_offsets(const GSArgs& k, uint64_t o, uint64_t& ao, uint64_t& co)
{
    ao = 0;
    co = 0;
    for (int m = 0; m < k.nm; ++m) {
        const uint64_t e = k.ext[m];
        const uint64_t q = o / e;
        const uint64_t d = o - q * e;
        ao += d * k.wa[m];
        co += d * k.wc[m];
        o = q;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) gs_col_kernel(GSArgs k)
{
    pdl_prologue();
    const T* __restrict__ A = static_cast<const T*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    constexpr int U = 8;
    for (uint64_t o = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; o < k.outputs;
         o += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t ao, co;
        gs_offsets(k, o, ao, co);
        Acc<T, true> acc;
        acc.init();
        uint64_t i = 0;
        for (; i + U <= k.nq; i += U) {
            T av[U];
#pragma unroll
            for (int u = 0; u < U; ++u) av[u] = A[ao + (i + u) * k.waq];
#pragma unroll
            for (int u = 0; u < U; ++u) acc.fma_add(av[u], __ldg(B + (i + u) * k.wb));
        }
        for (; i < k.nq; ++i) acc.fma_add(A[ao + i * k.waq], __ldg(B + i * k.wb));
        static_cast<T*>(k.c)[co] = acc.value();
    }
}

template <typename T>
__global__ void __launch_bounds__(256) gs_row_kernel(GSArgs k)
{
    pdl_prologue();
    const T* __restrict__ A = static_cast<const T*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    const uint32_t G = k.group;                 // lanes per output (power of two)
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gl = lane & (G - 1u);
    const uint64_t gid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / G;
    constexpr int U = 4;
    // every lane of a warp runs the same number of rounds (the shuffles below)
    const uint64_t rounds = (k.outputs + ngroups - 1) / ngroups;
    for (uint64_t r = 0; r < rounds; ++r) {
        const uint64_t o = gid + r * ngroups;
        const bool valid = o < k.outputs;
        Acc<T, true> acc;
        acc.init();
        uint64_t co = 0;
        if (valid) {
            uint64_t ao;
            gs_offsets(k, o, ao, co);
            uint64_t i = gl;
            for (; i + (uint64_t)G * (U - 1) < k.nq; i += (uint64_t)G * U) {
                T av[U];
#pragma unroll
                for (int u = 0; u < U; ++u) av[u] = A[ao + (i + (uint64_t)G * u) * k.waq];
#pragma unroll
                for (int u = 0; u < U; ++u) acc.fma_add(av[u], __ldg(B + (i + (uint64_t)G * u) * k.wb));
            }
            for (; i < k.nq; i += G) acc.fma_add(A[ao + i * k.waq], __ldg(B + i * k.wb));
        }
        for (uint32_t off = G >> 1; off > 0; off >>= 1) {
            const T os = __shfl_xor_sync(0xffffffffu, acc.s, off);
            const T oc = __shfl_xor_sync(0xffffffffu, acc.c, off);
            acc.merge(os, oc);
        }
        if (valid && gl == 0) static_cast<T*>(k.c)[co] = acc.value();
    }
}

// 16 bytes of b through the read-only path (16-byte aligned).
template <typename T, int V>
__device__ __forceinline__ void gs_load_b(const T* p, T (&out)[V])
{
    const uint4 r = __ldg(reinterpret_cast<const uint4*>(p));
    memcpy(out, &r, 16);
}

// 16-byte forms, where the views allow aligned vector loads (set by the host):
// row form with contiguous rows (wa[q] == 1, b contiguous, n_q and every row
// start on the 16-byte grid); column form with V consecutive outputs of A's
// fastest other mode (its stride 1, its extent and every other stride
// multiples of V, A on the 16-byte grid).
template <typename T>
__global__ void __launch_bounds__(256) gs_row_vec_kernel(GSArgs k)
{
    pdl_prologue();
    constexpr int V = 16 / (int)sizeof(T);
    constexpr int U = 4;
    const T* __restrict__ A = static_cast<const T*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    const uint32_t G = k.group;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gl = lane & (G - 1u);
    const uint64_t gid = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const uint64_t ngroups = ((uint64_t)gridDim.x * blockDim.x) / G;
    const uint64_t nv = k.nq / V;
    const uint64_t rounds = (k.outputs + ngroups - 1) / ngroups;
    for (uint64_t r = 0; r < rounds; ++r) {
        const uint64_t o = gid + r * ngroups;
        const bool valid = o < k.outputs;
        Acc<T, true> acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        uint64_t co = 0;
        if (valid) {
            uint64_t ao;
            gs_offsets(k, o, ao, co);
            const T* ap = A + ao;
            uint64_t kv = gl;
            for (; kv + (uint64_t)G * (U - 1) < nv; kv += (uint64_t)G * U) {
                T av[U][V], bv[U][V];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    load_a<T, T, V>(ap + (kv + (uint64_t)G * u) * V, av[u]);
                    gs_load_b<T, V>(B + (kv + (uint64_t)G * u) * V, bv[u]);
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v].fma_add(av[u][v], bv[u][v]);
            }
            for (; kv < nv; kv += G) {
                T av[V], bv[V];
                load_a<T, T, V>(ap + kv * V, av);
                gs_load_b<T, V>(B + kv * V, bv);
#pragma unroll
                for (int v = 0; v < V; ++v) acc[v].fma_add(av[v], bv[v]);
            }
        }
        fold_vec<V>(acc);
        for (uint32_t off = G >> 1; off > 0; off >>= 1) {
            const T os = __shfl_xor_sync(0xffffffffu, acc[0].s, off);
            const T oc = __shfl_xor_sync(0xffffffffu, acc[0].c, off);
            acc[0].merge(os, oc);
        }
        if (valid && gl == 0) static_cast<T*>(k.c)[co] = acc[0].value();
    }
}

template <typename T>
__global__ void __launch_bounds__(256) gs_col_vec_kernel(GSArgs k)
{
    pdl_prologue();
    constexpr int V = 16 / (int)sizeof(T);
    constexpr int U = 4;
    const T* __restrict__ A = static_cast<const T*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    const uint64_t groups = k.outputs / V;
    for (uint64_t og = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; og < groups;
         og += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t ao, co;
        gs_offsets(k, og * V, ao, co);
        Acc<T, true> acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        uint64_t i = 0;
        for (; i + U <= k.nq; i += U) {
            T av[U][V];
#pragma unroll
            for (int u = 0; u < U; ++u) load_a<T, T, V>(A + ao + (i + u) * k.waq, av[u]);
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const T bb = __ldg(B + (i + u) * k.wb);
#pragma unroll
                for (int v = 0; v < V; ++v) acc[v].fma_add(av[u][v], bb);
            }
        }
        for (; i < k.nq; ++i) {
            T av[V];
            load_a<T, T, V>(A + ao + i * k.waq, av);
            const T bb = __ldg(B + i * k.wb);
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v].fma_add(av[v], bb);
        }
        T* C = static_cast<T*>(k.c);
#pragma unroll
        for (int v = 0; v < V; ++v) C[co + (uint64_t)v * k.wc[0]] = acc[v].value();
    }
}

}  // namespace tlibg
