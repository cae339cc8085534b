// TTV kernels for sm_103a.
//
// Every layout of a dense tensor reduces to the canonical product
//     C[s, j] = sum_i A[s, i, j] * b[i],   A (S, nq, P) row-major, C (S, P),
// where P is the product of the extents laid out before mode q, nq = n_q and
// S the product of the extents after it (the reference's "subtensor" view,
// tensor_times_vector.h:1208-1256, with all free modes fused, fusion::all).
//
//  row_kernel  (P == 1, q is the fastest mode; the reference's gemv_row /
//              dot, matrix_times_vector.h:52-91,265-295): a group of G lanes
//              (1..32) owns one row segment, streams it with 16-byte loads
//              and reduces with warp shuffles.
//  col_kernel  (P > 1; the reference's gemv_col over subtensors,
//              matrix_times_vector.h:109-221): each thread owns V consecutive
//              outputs of the contiguous prefix, warps are stacked along i
//              (WI per CTA) and reduced through shared memory; the b segment
//              of the CTA's work is staged in shared memory by a TMA bulk copy.
//  combine_kernel: deterministic second phase of the split-n_q reduction,
//              partials summed in a fixed order (fp64 for long fp32 rows).
//
// Both main kernels are HBM-streaming: A is read exactly once with
// evict-first loads, C written once.
#include "ttv_device.cuh"
#include "ttv_kernels.cuh"

#include <algorithm>
#include <mutex>
#include <type_traits>
#include <unordered_map>
#include <utility>

namespace tlibg {

static __device__ unsigned int g_device_error = 0u;

template <typename T> struct Pair {
    T s, c;
};

// Independent loads each thread keeps in flight: 4 of 16 bytes, or
// TLIBG_NARROW_INFLIGHT bytes (at most 16 loads) for narrower loads, so
// misaligned or odd-extent layouts still cover the HBM latency-bandwidth
// product.
// Resident CTAs per SM the register kernels are compiled for (the
// __launch_bounds__ minimum): 4 for 16-byte loads, 1 for narrower ones.
// Measured on GB300 over the symmetric sweep against other targets (1, 4, 5,
// 6) and against no minimum: column fp32 V4 5.92 -> 6.57 TB/s, fp64 V2
// 6.19 -> 6.25, row fp32 V4 6.05 -> 6.46; narrow loads lose with 4.
template <typename TA, int V> __host__ __device__ constexpr int min_ctas()
{
    return (int)sizeof(TA) * V >= 16 ? 4 : 1;
}

// Narrow loads: 64 bytes in flight (at most 16 loads).  Measured on GB300 over
// the symmetric sweep: rows of 645 doubles (fp64 scalar loads, 8 in flight)
// 5.70 TB/s against 5.31 with 128 bytes (16 loads: 111 registers, 2 CTAs per
// SM), 4.73 with 96 and 5.16 with 32; rows of 645 floats 5.72 with 64 or 128
// bytes (16 loads either way), 5.25 with 32.
#ifndef TLIBG_NARROW_INFLIGHT
#define TLIBG_NARROW_INFLIGHT 64
#endif
template <typename TA, int V> __host__ __device__ constexpr int loads_in_flight()
{
    return (int)sizeof(TA) * V >= 16 ? 4
           : (TLIBG_NARROW_INFLIGHT / ((int)sizeof(TA) * V) > 16 ? 16 : TLIBG_NARROW_INFLIGHT / ((int)sizeof(TA) * V));
}

// --------------------------------------------------------------------------
// vector load of b (V elements of T, aligned), via the read-only path
// --------------------------------------------------------------------------
template <typename T, int V>
__device__ __forceinline__ void load_b(const T* p, T (&out)[V])
{
    constexpr int B = (int)sizeof(T) * V;
    if constexpr (B <= 16) {
        typedef typename RawVec<B < 4 ? 4 : B>::type R;
        if constexpr (B >= 4) {
            R r = __ldg(reinterpret_cast<const R*>(p));
            const T* e = reinterpret_cast<const T*>(&r);
#pragma unroll
            for (int v = 0; v < V; ++v) out[v] = e[v];
        }
    } else {
        // 32 bytes: two 16-byte loads
        uint4 r0 = __ldg(reinterpret_cast<const uint4*>(p));
        uint4 r1 = __ldg(reinterpret_cast<const uint4*>(p) + 1);
        const T* e0 = reinterpret_cast<const T*>(&r0);
        const T* e1 = reinterpret_cast<const T*>(&r1);
        constexpr int H = 16 / (int)sizeof(T);
#pragma unroll
        for (int v = 0; v < H; ++v) out[v] = e0[v];
#pragma unroll
        for (int v = 0; v < H; ++v) out[H + v] = e1[v];
    }
}

// acc[v] += av[v] * bb for the V outputs of one thread.  With the fp64
// double-float accumulator the work is mixed: half the products take a native
// DFMA (even outputs, or even unrolled rows when V == 1) and half the FP32 /
// INT32 emulation, so neither the FP64 pipe nor the issue slots alone bound
// the kernel; the shared bb is split once.
// One product in TLIBG_F64_NATIVE_EVERY (counted over the unrolled loads and
// vector slots) takes the DFMA pipe, the others the double-float emulation.
// Measured on GB300 over the symmetric sweep's fp64 half: one in two is best
// (one in three or four, or all but one in three or four, lose 3-14 %).
#ifndef TLIBG_F64_NATIVE_EVERY
#define TLIBG_F64_NATIVE_EVERY 2
#endif
template <int V> __device__ __forceinline__ constexpr bool f64_native(int u, int v)
{
    return ((u * V + v) % TLIBG_F64_NATIVE_EVERY) == 0;
}

// bsp (PRE): b's double-float split, computed once per staged segment.
template <int V, bool PRE = false, typename AccT, typename T>
__device__ __forceinline__ void row_fma(AccT (&acc)[V], const T (&av)[V], T bb, int u = 0,
                                        const float2* bsp = nullptr)
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
        for (int v = 0; v < V; ++v) {
            const bool native = f64_native<V>(u, v);
            if (native)
                acc[v].d = fma(av[v], bb, acc[v].d);
            else
                acc[v].add_split(split_double(av[v]), bs, av[v], bb);
        }
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].fma_add(av[v], bb);
    }
}

// acc[v] += av[v] * bv[v] (row form: b varies with the element).  The fp64
// double-float accumulator mixes the same way: even vector slots (or even
// unrolled loads when V == 1) on the DFMA pipe, odd ones emulated.
template <int V, bool PRE = false, typename AccT, typename T>
__device__ __forceinline__ void vec_fma(AccT (&acc)[V], const T (&av)[V], const T (&bv)[V], int u = 0,
                                        const float2* bsp = nullptr)
{
    if constexpr (std::is_same<AccT, AccDF>::value) {
#pragma unroll
        for (int v = 0; v < V; ++v) {
            const bool native = f64_native<V>(u, v);
            if (native) {
                acc[v].d = fma(av[v], bv[v], acc[v].d);
            } else if constexpr (PRE) {
                const float2 t = bsp[v];
                DSplit bs;
                bs.hi = t.x;
                bs.lo = t.y;
                bs.ok = true;
                acc[v].add_split(split_double(av[v]), bs, av[v], bv[v]);
            } else {
                acc[v].add_split(split_double(av[v]), split_double(bv[v]), av[v], bv[v]);
            }
        }
    } else {
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].fma_add(av[v], bv[v]);
    }
}

template <int V, typename AccT> __device__ __forceinline__ void renorm_all(AccT (&acc)[V])
{
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v].renorm();
}

// UB rows of the contracted mode for one thread: all loads first, then the
// products (column form: b[i] shared by the V outputs; u alternates the fp64
// mix when V == 1).
// rp points at the thread's vector in row i and moves on by `step` elements
// (WI rows) per row: one pointer add per load.
template <int UB, int V, bool PRE = false, typename TA, typename T, typename AccT>
__device__ __forceinline__ void col_rows(AccT (&acc)[V], const TA*& rp, uint64_t step, const T* bs, uint64_t i,
                                         uint32_t WI, const float2* bsp = nullptr)
{
    T av[UB][V];
#pragma unroll
    for (int u = 0; u < UB; ++u) {
        load_a<TA, T, V>(rp, av[u]);
        rp += step;
    }
#pragma unroll
    for (int u = 0; u < UB; ++u) row_fma<V, PRE>(acc, av[u], bs[i + u * WI], u, PRE ? bsp + i + u * WI : nullptr);
    renorm_all<V>(acc);
}

// Rows [i0, ie) step WI of one thread: blocks of U rows, then one of U/2 and
// one of U/4 at most, then single rows, so short contractions still get
// their loads in flight together.
template <int U, int V, bool PRE, typename TA, typename T, typename AccT>
__device__ __forceinline__ void col_loop(AccT (&acc)[V], const TA* ap, uint64_t P, const T* bs, const float2* bsp,
                                         uint64_t i, uint64_t ie, uint32_t WI)
{
    const TA* rp = ap + i * P;
    const uint64_t step = uint64_t(WI) * P;
    for (; i + (U - 1) * WI < ie; i += U * WI) col_rows<U, V, PRE>(acc, rp, step, bs, i, WI, bsp);
    if constexpr (U >= 4) {
        if (i + (U / 2 - 1) * WI < ie) {
            col_rows<U / 2, V, PRE>(acc, rp, step, bs, i, WI, bsp);
            i += (U / 2) * WI;
        }
    }
    if constexpr (U >= 8) {
        if (i + (U / 4 - 1) * WI < ie) {
            col_rows<U / 4, V, PRE>(acc, rp, step, bs, i, WI, bsp);
            i += (U / 4) * WI;
        }
    }
    for (; i < ie; i += WI) col_rows<1, V, PRE>(acc, rp, step, bs, i, WI, bsp);
}

// fp64 with the double-float mix: b's split is computed once per staged
// segment (shared by every tile of the CTA) instead of once per row and thread.
template <typename T, bool KAHAN> __host__ __device__ constexpr bool presplit_b()
{
    return std::is_same<T, double>::value && KAHAN;
}

// Split the staged segment b[0..n) into bsp; true (CTA-uniform) when every
// element is inside the emulation's exponent window.
template <typename T>
__device__ __forceinline__ bool stage_b_split(const T* b, uint32_t n, float2* bsp)
{
    int ok = 1;
    if constexpr (std::is_same<T, double>::value) {
        for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
            const DSplit d = split_double(b[e]);
            bsp[e] = make_float2(d.hi, d.lo);
            ok &= d.ok ? 1 : 0;
        }
    }
    return __syncthreads_and(ok) != 0;
}

// Same for UB vectors of a row (row form: b varies with the element).
template <int UB, int V, bool PRE = false, typename TA, typename T, typename AccT>
__device__ __forceinline__ void row_vecs(AccT (&acc)[V], const TA* ap, const T* bp, uint64_t kv, uint32_t G,
                                         const float2* bsp = nullptr)
{
    T av[UB][V], bv[UB][V];
#pragma unroll
    for (int u = 0; u < UB; ++u) {
        if (G == 1)   // one lane per row: keep the sector's other half in L1
            load_a_l1<TA, T, V>(ap + (kv + u) * V, av[u]);
        else
            load_a<TA, T, V>(ap + (kv + u * G) * V, av[u]);
        load_b<T, V>(bp + (kv + u * G) * V, bv[u]);
    }
#pragma unroll
    for (int u = 0; u < UB; ++u) vec_fma<V, PRE>(acc, av[u], bv[u], u, PRE ? bsp + (kv + u * G) * V : nullptr);
    renorm_all<V>(acc);
}

// One row segment [0, nv) vectors of a lane (kv = gl, gl + G, ...).
template <int U, int V, bool PRE, typename TA, typename T, typename AccT>
__device__ __forceinline__ void row_loop(AccT (&acc)[V], const TA* ap, const T* bp, const float2* bsp, uint64_t kv,
                                         uint64_t nv, uint32_t G)
{
    // blocks of U vectors, then one of U/2 and one of U/4 at most, then
    // single vectors: short rows still get their loads in flight together
    for (; kv + (U - 1) * G < nv; kv += U * G) row_vecs<U, V, PRE>(acc, ap, bp, kv, G, bsp);
    if constexpr (U >= 4) {
        if (kv + (U / 2 - 1) * G < nv) {
            row_vecs<U / 2, V, PRE>(acc, ap, bp, kv, G, bsp);
            kv += (U / 2) * G;
        }
    }
    if constexpr (U >= 8) {
        if (kv + (U / 4 - 1) * G < nv) {
            row_vecs<U / 4, V, PRE>(acc, ap, bp, kv, G, bsp);
            kv += (U / 4) * G;
        }
    }
    for (; kv < nv; kv += G) row_vecs<1, V, PRE>(acc, ap, bp, kv, G, bsp);
}

// fp64 rows with the double-float mix: b (up to this many elements) is split
// once per CTA into shared memory.
constexpr int ROW_SPLIT_MAX = 2048;

// --------------------------------------------------------------------------
// row kernel: P == 1
// --------------------------------------------------------------------------

// Short rows (n_q a multiple of V, at most M vectors per lane of a group, no
// split): a lane's M vectors of b are the same for every row and loaded once;
// each iteration loads M vectors of each of R rows before any product, so a
// row of a few dozen elements still keeps R * M loads per lane in flight.
// Missing vectors (n_q / V not a multiple of G) are zeros, which add nothing.
template <int M, int R, typename TA, typename T, int V, bool KAHAN>
__device__ __forceinline__ void row_short(const KArgs& k, uint32_t G, uint32_t lane, uint64_t warp_id,
                                          uint64_t nwarps)
{
    const uint32_t gl = lane & (G - 1u);
    const uint32_t gpw = 32u / G;
    const uint64_t nv = k.nq / V;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    T bv[M][V];
#pragma unroll
    for (int t = 0; t < M; ++t) {
        const uint64_t kv = gl + (uint64_t)t * G;
        if (kv < nv) {
            load_b<T, V>(B + kv * V, bv[t]);
        } else {
#pragma unroll
            for (int v = 0; v < V; ++v) bv[t][v] = T(0);
        }
    }
    const uint64_t per_iter = (uint64_t)gpw * R;
    for (uint64_t base = warp_id * per_iter; base < k.items; base += nwarps * per_iter) {
        T av[R][M][V];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint64_t item = base + (uint64_t)r * gpw + lane / G;
#pragma unroll
            for (int t = 0; t < M; ++t) {
                const uint64_t kv = gl + (uint64_t)t * G;
                if (item < k.items && kv < nv) {
                    load_a<TA, T, V>(A + item * k.nq + kv * V, av[r][t]);
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v) av[r][t][v] = T(0);
                }
            }
        }
#pragma unroll
        for (int r = 0; r < R; ++r) {
            const uint64_t item = base + (uint64_t)r * gpw + lane / G;
            typename AccSel<T, KAHAN>::type acc[V];
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v].init();
#pragma unroll
            for (int t = 0; t < M; ++t) vec_fma<V>(acc, av[r][t], bv[t], t);
            renorm_all<V>(acc);
            fold_vec<V>(acc);
            for (uint32_t off = G >> 1; off > 0; off >>= 1) {
                T os = __shfl_xor_sync(0xffffffffu, acc[0].s, off);
                T oc = __shfl_xor_sync(0xffffffffu, acc[0].c, off);
                acc[0].merge(os, oc);
            }
            if (item < k.items && gl == 0) static_cast<T*>(k.out)[item] = acc[0].value();
        }
    }
}

template <typename TA, typename T, int V, bool KAHAN>
__global__ void __launch_bounds__(BLOCK, (min_ctas<TA, V>())) row_kernel(KArgs k)
{
    pdl_prologue();
    const uint32_t G = k.group;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t gl = lane & (G - 1u);
    const uint32_t gpw = 32u / G;
    const uint64_t warp_id = (uint64_t(blockIdx.x) * BLOCK + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * BLOCK) >> 5;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    constexpr int U = loads_in_flight<TA, V>();
    constexpr bool PRES = presplit_b<T, KAHAN>();
    extern __shared__ __align__(16) unsigned char row_smem[];
    float2* bsplit = reinterpret_cast<float2*>(row_smem);
    bool b_split_ok = false;
    if constexpr (PRES) {
        // the planner gives this kernel ROW_SPLIT_MAX float2 of shared memory (not
        // with one lane per row: those rows live off L1, which shared memory shrinks)
        if (k.nq <= (uint64_t)ROW_SPLIT_MAX && G > 1) b_split_ok = stage_b_split<T>(B, (uint32_t)k.nq, bsplit);
    }

    for (uint64_t wbase = warp_id * gpw; wbase < k.items; wbase += nwarps * gpw) {
        const uint64_t item = wbase + lane / G;
        const bool valid = item < k.items;
        typename AccSel<T, KAHAN>::type acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        uint64_t row = 0, seg = 0;
        if (valid) {
            if (k.nseg == 1) {
                row = item;
            } else {
                // segment-major: the rows' pieces of one b segment are taken up
                // together, so b (as long as a row) is read from HBM about once
                seg = item / k.S;
                row = item - seg * k.S;
            }
            const uint64_t ib = seg * k.seg_len;
            const uint64_t ie = min(k.nq, ib + k.seg_len);
            const TA* ap = A + row * k.nq + ib;
            const T* bp = B + ib;
            const uint64_t n = ie - ib;
            const uint64_t nv = n / V;
            if constexpr (PRES) {
                if (b_split_ok)
                    row_loop<U, V, true>(acc, ap, bp, bsplit + ib, gl, nv, G);
                else
                    row_loop<U, V, false>(acc, ap, bp, bsplit, gl, nv, G);
            } else {
                row_loop<U, V, false>(acc, ap, bp, bsplit, gl, nv, G);
            }
            for (uint64_t e = nv * V + gl; e < n; e += G) {
                T av[1];
                load_a<TA, T, 1>(ap + e, av);
                acc[0].fma_add(av[0], __ldg(bp + e));
            }
        }
        fold_vec<V>(acc);
        for (uint32_t off = G >> 1; off > 0; off >>= 1) {
            T os = __shfl_xor_sync(0xffffffffu, acc[0].s, off);
            T oc = __shfl_xor_sync(0xffffffffu, acc[0].c, off);
            acc[0].merge(os, oc);
        }
        if (valid && gl == 0) {
            if (k.nseg == 1) {
                static_cast<T*>(k.out)[row] = acc[0].value();
            } else {
                Pair<T> pr;
                pr.s = acc[0].s;
                pr.c = KAHAN ? acc[0].c : T(0);
                static_cast<Pair<T>*>(k.partial)[seg * k.S + row] = pr;
            }
        }
    }
}

// Column form with a contraction of at most CS_MAXQ rows (no split, vector
// loads): one round of the column kernel's tile loop would keep only n_q
// loads in flight per thread, one HBM round trip per tile.  Here each thread
// owns V consecutive outputs in each of two tiles TO apart and loads every row
// of both before any product: 2 n_q vector loads in flight per thread.  b's
// n_q values (and for fp64 their split) live in registers.
#ifndef TLIBG_CS_VSTORE
#define TLIBG_CS_VSTORE 1
#endif
template <typename TA, typename T, int V, bool KAHAN>
__global__ void __launch_bounds__(BLOCK, (min_ctas<TA, V>())) col_short_kernel(KArgs k)
{
    pdl_prologue();
    constexpr bool PRES = presplit_b<T, KAHAN>();
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    const uint32_t nq = (uint32_t)k.nq;
    const uint64_t P = k.P;
    const uint64_t outputs = k.S * P;
    constexpr uint64_t TO = (uint64_t)BLOCK * V;
    T bq[CS_MAXQ];
    float2 bsp[CS_MAXQ];
    bool split_ok = true;
#pragma unroll
    for (int i = 0; i < CS_MAXQ; ++i) {
        bq[i] = (uint32_t)i < nq ? __ldg(B + i) : T(0);
        if constexpr (PRES) {
            const DSplit d = split_double((double)bq[i]);
            bsp[i] = make_float2(d.hi, d.lo);
            split_ok = split_ok && (d.ok || (uint32_t)i >= nq);
        }
    }
    const uint64_t first = uint64_t(blockIdx.x) * k.items_per_cta;
    const uint64_t last = min(k.items, first + k.items_per_cta);
    for (uint64_t pair = first; pair < last; ++pair) {
        T av[2][CS_MAXQ][V];
        bool valid[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const uint64_t o = (2 * pair + h) * TO + (uint64_t)threadIdx.x * V;
            valid[h] = o < outputs;
            const uint64_t s = valid[h] ? idx_div(o, k.pdiv) : 0;
            const TA* ap = A + (s * k.nq) * P + (o - s * P);
#pragma unroll
            for (int i = 0; i < CS_MAXQ; ++i) {
                if (valid[h] && (uint32_t)i < nq) {
                    load_a<TA, T, V>(ap + (uint64_t)i * P, av[h][i]);
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v) av[h][i][v] = T(0);
                }
            }
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            typename AccSel<T, KAHAN>::type acc[V];
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v].init();
#pragma unroll
            for (int i = 0; i < CS_MAXQ; ++i) {
                if ((uint32_t)i < nq) {
                    if constexpr (PRES) {
                        if (split_ok)
                            row_fma<V, true>(acc, av[h][i], bq[i], i, &bsp[i]);
                        else
                            row_fma<V, false>(acc, av[h][i], bq[i], i, nullptr);
                    } else {
                        row_fma<V, false>(acc, av[h][i], bq[i], i, nullptr);
                    }
                }
            }
            renorm_all<V>(acc);
            if (valid[h]) {
                const uint64_t o = (2 * pair + h) * TO + (uint64_t)threadIdx.x * V;
                T vals[V];
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    acc[v].fold();
                    vals[v] = acc[v].value();
                }
                T* out = static_cast<T*>(k.out) + o;
                // C is a quarter of A or more here: one vector store per thread where aligned
                constexpr int VB = V * (int)sizeof(T);
                bool vec_done = false;
                if constexpr (VB <= 16 && TLIBG_CS_VSTORE) {
                    if (o + V <= outputs && (reinterpret_cast<uintptr_t>(out) % VB) == 0) {
                        typedef typename RawVec<VB>::type R;
                        R r;
                        memcpy(&r, vals, sizeof(R));
                        *reinterpret_cast<R*>(out) = r;
                        vec_done = true;
                    }
                }
                if (!vec_done) {
#pragma unroll
                    for (int v = 0; v < V; ++v)
                        if (o + v < outputs) out[v] = vals[v];
                }
            }
        }
    }
}

// Short rows as their own kernel (its registers do not weigh on the general
// row kernel): M vectors per lane of each row, R = U / M rows in flight.
template <typename TA, typename T, int V, bool KAHAN, int M>
__global__ void __launch_bounds__(BLOCK, (min_ctas<TA, V>())) row_short_kernel(KArgs k)
{
    pdl_prologue();
    constexpr int U = loads_in_flight<TA, V>();
    constexpr int R = M == 1 ? U : (U >= 2 ? U / 2 : 1);
    const uint64_t warp_id = (uint64_t(blockIdx.x) * BLOCK + threadIdx.x) >> 5;
    const uint64_t nwarps = (uint64_t(gridDim.x) * BLOCK) >> 5;
    row_short<M, R, TA, T, V, KAHAN>(k, k.group, threadIdx.x & 31u, warp_id, nwarps);
}

// --------------------------------------------------------------------------
// column kernel: P > 1
// --------------------------------------------------------------------------
template <typename TA, typename T, int V, bool KAHAN>
__global__ void __launch_bounds__(BLOCK, (min_ctas<TA, V>())) col_kernel(KArgs k)
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

    const uint32_t WI = k.group;
    const uint32_t WO = (BLOCK / 32) / WI;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t wi = warp % WI, wo = warp / WI;
    const uint64_t TO = uint64_t(WO) * 32u * V;
    const uint64_t outputs = k.S * k.P;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);
    const T* __restrict__ B = static_cast<const T*>(k.b);
    constexpr int U = loads_in_flight<TA, V>();
    bool b_split_ok = false;

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

        const uint64_t o0 = tile * TO + (uint64_t(wo) * 32u + lane) * V;
        const bool valid = o0 < outputs;
        typename AccSel<T, KAHAN>::type acc[V];
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].init();
        if (valid) {
            const uint64_t s = idx_div(o0, k.pdiv);
            const uint64_t j = o0 - s * k.P;
            const TA* ap = A + (s * k.nq) * k.P + j;
            if constexpr (PRES) {
                if (b_split_ok)
                    col_loop<U, V, true>(acc, ap, k.P, bs, bsp, ib + wi, ie, WI);
                else
                    col_loop<U, V, false>(acc, ap, k.P, bs, bsp, ib + wi, ie, WI);
            } else {
                col_loop<U, V, false>(acc, ap, k.P, bs, bsp, ib + wi, ie, WI);
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v) acc[v].fold();
        if (WI > 1) {
            // warps stacked along i hand their partials to warp row wi == 0
            const uint32_t slot = wo * 32u + lane;
            if (wi > 0) {
                T* r = red + ((size_t)(wi - 1) * (WO * 32u) + slot) * (2 * V);
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    r[2 * v] = acc[v].s;
                    r[2 * v + 1] = acc[v].c;
                }
            }
            __syncthreads();
            if (wi == 0) {
                for (uint32_t w = 1; w < WI; ++w) {
                    const T* r = red + ((size_t)(w - 1) * (WO * 32u) + slot) * (2 * V);
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[v].merge(r[2 * v], r[2 * v + 1]);
                }
            }
            __syncthreads();
        }
        if (wi == 0 && valid) {
            if (k.nseg == 1) {
                T* out = static_cast<T*>(k.out) + o0;
                const bool vec_ok = ((reinterpret_cast<uintptr_t>(out) % (sizeof(T) * V)) == 0) &&
                                    (sizeof(T) * V <= 16);
                if (vec_ok && V > 1) {
                    T vals[V];
#pragma unroll
                    for (int v = 0; v < V; ++v) vals[v] = acc[v].value();
                    if constexpr (sizeof(T) * V == 16) {
                        *reinterpret_cast<uint4*>(out) = *reinterpret_cast<const uint4*>(vals);
                    } else if constexpr (sizeof(T) * V == 8) {
                        *reinterpret_cast<uint2*>(out) = *reinterpret_cast<const uint2*>(vals);
                    } else {
#pragma unroll
                        for (int v = 0; v < V; ++v) out[v] = vals[v];
                    }
                } else {
#pragma unroll
                    for (int v = 0; v < V; ++v) out[v] = acc[v].value();
                }
            } else {
                Pair<T>* pp = static_cast<Pair<T>*>(k.partial) + seg * outputs + o0;
#pragma unroll
                for (int v = 0; v < V; ++v) {
                    Pair<T> pr;
                    pr.s = acc[v].s;
                    pr.c = KAHAN ? acc[v].c : T(0);
                    pp[v] = pr;
                }
            }
        }
    }
}

// --------------------------------------------------------------------------
// combine kernel: C[o] = sum over segments of partial[seg][o], fixed order
// --------------------------------------------------------------------------
// tpo threads per output (a power of two): thread t sums segments t, t + tpo,
// ... in order, loading COMBINE_U of them before the first sum so their
// latencies overlap; then the tpo partial sums meet in a fixed tree (pairs
// (t, t + h) for h = tpo/2 .. 1: through shared memory while h spans warps,
// by warp shuffles below), so the result is the same on every run.  Few
// outputs with many segments (thin prefixes, long contractions) spread over
// the whole block.
constexpr int COMBINE_U = 8;

template <typename T, bool KAHAN, bool F64>
__global__ void __launch_bounds__(BLOCK) combine_kernel(const Pair<T>* __restrict__ part,
                                                        T* __restrict__ out, uint64_t outputs,
                                                        uint32_t nseg, uint32_t tpo)
{
    pdl_prologue();
    __shared__ double red[2 * BLOCK];
    const uint32_t t = threadIdx.x & (tpo - 1u);
    const uint32_t ob = threadIdx.x / tpo;
    const uint32_t opb = BLOCK / tpo;
    for (uint64_t base = uint64_t(blockIdx.x) * opb; base < outputs; base += uint64_t(gridDim.x) * opb) {
        const uint64_t o = base + ob;
        double fs = 0.0;                 // F64: plain double sum
        Acc<T, KAHAN> acc;               // else: compensated merge of (s, c) pairs
        acc.init();
        if (o < outputs) {
            for (uint32_t g0 = t; g0 < nseg; g0 += COMBINE_U * tpo) {
                Pair<T> pv[COMBINE_U];
#pragma unroll
                for (int u = 0; u < COMBINE_U; ++u) {
                    const uint32_t g = g0 + (uint32_t)u * tpo;
                    if (g < nseg) {
                        pv[u] = part[uint64_t(g) * outputs + o];
                    } else {
                        pv[u].s = T(0);
                        pv[u].c = T(0);
                    }
                }
#pragma unroll
                for (int u = 0; u < COMBINE_U; ++u) {
                    if (g0 + (uint32_t)u * tpo < nseg) {
                        if (F64)
                            fs += (double)pv[u].s - (double)pv[u].c;
                        else
                            acc.merge(pv[u].s, pv[u].c);
                    }
                }
            }
        }
        if (tpo > 1) {
            uint32_t h = tpo >> 1;
            for (; h >= 32; h >>= 1) {
                red[2 * threadIdx.x] = F64 ? fs : (double)acc.s;
                red[2 * threadIdx.x + 1] = F64 ? 0.0 : (double)acc.c;
                __syncthreads();
                if (t < h) {
                    const double os = red[2 * (threadIdx.x + h)], oc = red[2 * (threadIdx.x + h) + 1];
                    if (F64)
                        fs += os;
                    else
                        acc.merge((T)os, (T)oc);
                }
                __syncthreads();
            }
            // the rest of the tree inside a warp (a group of tpo <= 32 lanes, or the
            // first warp of a larger group)
            for (; h > 0; h >>= 1) {
                if (F64) {
                    const double os = __shfl_down_sync(0xffffffffu, fs, h);
                    if (t < h) fs += os;
                } else {
                    const T os = __shfl_down_sync(0xffffffffu, acc.s, h);
                    const T oc = __shfl_down_sync(0xffffffffu, acc.c, h);
                    if (t < h) acc.merge(os, oc);
                }
            }
        }
        if (t == 0 && o < outputs) out[o] = F64 ? (T)fs : acc.value();
    }
}

}  // namespace tlibg

#include "ttv_stream.cuh"
#include "ttv_realign.cuh"
#include "ttv_thin.cuh"
#include "ttv_strided.cuh"
#include "ttv_rowtile.cuh"
#include "ttv_colbulk.cuh"
#include "ttv_rowpanel.cuh"
#include "ttv_rowshift.cuh"

namespace tlibg {

// --------------------------------------------------------------------------
// host side: instantiation tables
// --------------------------------------------------------------------------
typedef void (*KernelFn)(KArgs);

template <typename TA, typename T, int M, bool KAHAN>
static KernelFn pick_short(int vec)
{
    constexpr int VMAX = 16 / (int)sizeof(TA);
    switch (vec) {
    case 1: return row_short_kernel<TA, T, 1, KAHAN, M>;
    case 2: return row_short_kernel<TA, T, 2, KAHAN, M>;
    case 4: if constexpr (VMAX >= 4) return row_short_kernel<TA, T, 4, KAHAN, M>; else return nullptr;
    case 8: if constexpr (VMAX >= 8) return row_short_kernel<TA, T, 8, KAHAN, M>; else return nullptr;
    }
    return nullptr;
}

template <typename TA, typename T, bool KAHAN>
static KernelFn pick_main(int kind, int vec, int rows_m, int mo)
{
    constexpr int VMAX = 16 / (int)sizeof(TA);
    if (kind == KIND_COL_BULK) return col_bulk_kernel<TA, T, KAHAN>;
    if (kind == KIND_ROW_SHIFT) {
        if constexpr (std::is_same<TA, T>::value) return row_shift_kernel<T, KAHAN>;
        else return nullptr;
    }
    if (kind == KIND_ROW_PANEL) {
        if (vec != VMAX) return nullptr;
        return rows_m == 2 ? row_panel_kernel<TA, T, VMAX, KAHAN, 2> : row_panel_kernel<TA, T, VMAX, KAHAN, 1>;
    }
    if (kind == KIND_ROW_TILE) {
        switch (rows_m) {
        case 1: return row_tile_kernel<TA, T, KAHAN, 1>;
        case 2: return row_tile_kernel<TA, T, KAHAN, 2>;
        case 4: return row_tile_kernel<TA, T, KAHAN, 4>;
        }
        return nullptr;
    }
    if (kind == KIND_COL && rows_m == 1 && vec > 1) {
        switch (vec) {
        case 2: return col_short_kernel<TA, T, 2, KAHAN>;
        case 4: if constexpr (VMAX >= 4) return col_short_kernel<TA, T, 4, KAHAN>; else return nullptr;
        case 8: if constexpr (VMAX >= 8) return col_short_kernel<TA, T, 8, KAHAN>; else return nullptr;
        }
        return nullptr;
    }
    if (kind == KIND_COL && vec == 1 && mo == 2) return col_strided_kernel<TA, T, 2, KAHAN>;
    if (kind == KIND_COL && vec == 1 && mo == 4) return col_strided_kernel<TA, T, 4, KAHAN>;
    if (kind == KIND_COL_REALIGN) {
        if constexpr (std::is_same<TA, T>::value) return col_realign_kernel<T, KAHAN>;
        else return nullptr;
    }
    if (kind == KIND_COL_THIN) {
        switch (vec) {
        case 1: return col_thin_kernel<TA, T, 1, KAHAN>;
        case 2: return col_thin_kernel<TA, T, 2, KAHAN>;
        case 4: if constexpr (VMAX >= 4) return col_thin_kernel<TA, T, 4, KAHAN>; else return nullptr;
        case 8: if constexpr (VMAX >= 8) return col_thin_kernel<TA, T, 8, KAHAN>; else return nullptr;
        }
        return nullptr;
    }
    if (kind == KIND_ROW && rows_m == 1) return pick_short<TA, T, 1, KAHAN>(vec);
    if (kind == KIND_ROW && rows_m == 2) return pick_short<TA, T, 2, KAHAN>(vec);
    if (kind == KIND_ROW) {
        switch (vec) {
        case 1: return row_kernel<TA, T, 1, KAHAN>;
        case 2: return row_kernel<TA, T, 2, KAHAN>;
        case 4: if constexpr (VMAX >= 4) return row_kernel<TA, T, 4, KAHAN>; else return nullptr;
        case 8: if constexpr (VMAX >= 8) return row_kernel<TA, T, 8, KAHAN>; else return nullptr;
        }
    } else {
        switch (vec) {
        case 1: return col_kernel<TA, T, 1, KAHAN>;
        case 2: return col_kernel<TA, T, 2, KAHAN>;
        case 4: if constexpr (VMAX >= 4) return col_kernel<TA, T, 4, KAHAN>; else return nullptr;
        case 8: if constexpr (VMAX >= 8) return col_kernel<TA, T, 8, KAHAN>; else return nullptr;
        }
    }
    return nullptr;
}

typedef void (*StreamFn)(SArgs);

static StreamFn stream_fn(const Plan& p)
{
    const bool col = p.stream_col != 0;
    switch (p.dtype) {
    case F32:
        if (p.kahan) return col ? stream_kernel<float, float, true, true> : stream_kernel<float, float, true, false>;
        return col ? stream_kernel<float, float, false, true> : stream_kernel<float, float, false, false>;
    case F64:
        if (p.kahan) return col ? stream_kernel<double, double, true, true> : stream_kernel<double, double, true, false>;
        return col ? stream_kernel<double, double, false, true> : stream_kernel<double, double, false, false>;
    case BF16A:
        if (p.kahan)
            return col ? stream_kernel<uint16_t, float, true, true> : stream_kernel<uint16_t, float, true, false>;
        return col ? stream_kernel<uint16_t, float, false, true> : stream_kernel<uint16_t, float, false, false>;
    }
    return nullptr;
}

bool stream_eligible(int dtype, uint64_t P, uint64_t nq)
{
    const uint64_t ea = dtype == F64 ? 8 : (dtype == BF16A ? 2 : 4);
    if (P == 1) return nq * ea <= (uint64_t)STREAM_STAGE;
    return P * ea <= (uint64_t)STREAM_STAGE && (P + STREAM_NT - 1) / STREAM_NT <= (uint64_t)STREAM_MAXJ;
}

// The kernel of a plan that takes KArgs (every kind but the streamed one).
static KernelFn main_kernel(const Plan& p)
{
    if (p.kind == KIND_STREAM) return nullptr;
    switch (p.dtype) {
    case F32:
        return p.kahan ? pick_main<float, float, true>(p.kind, p.vec, p.rows_m, p.mo)
                       : pick_main<float, float, false>(p.kind, p.vec, p.rows_m, p.mo);
    case F64:
        return p.kahan ? pick_main<double, double, true>(p.kind, p.vec, p.rows_m, p.mo)
                       : pick_main<double, double, false>(p.kind, p.vec, p.rows_m, p.mo);
    case BF16A:
        return p.kahan ? pick_main<uint16_t, float, true>(p.kind, p.vec, p.rows_m, p.mo)
                       : pick_main<uint16_t, float, false>(p.kind, p.vec, p.rows_m, p.mo);
    }
    return nullptr;
}

static size_t acc_size(int dtype) { return dtype == F64 ? 8 : 4; }

size_t plan_smem_bytes(const Plan& p)
{
    if (p.kind == KIND_STREAM) {
        const size_t es = acc_size(p.dtype);
        size_t extra = 2 * (size_t)STREAM_NT * es;
        if (!p.stream_col) extra = std::max(extra, (size_t)p.L * es);
        return 128 + (size_t)STREAM_NS * STREAM_SLOT + extra;
    }
    if (p.kind == KIND_COL_BULK) return 128 + (size_t)CB_NS * CB_STAGE_AL;
    if (p.kind == KIND_ROW_TILE) {
        const size_t ea = p.dtype == F64 ? 8 : (p.dtype == BF16A ? 2 : 4);
        return 128 + rowt_b_bytes(p.nq, acc_size(p.dtype)) + rowt_split_bytes(p.nq, p.dtype == F64 && p.kahan) +
               (size_t)ROWT_WARPS * ROWT_NS * rowt_slot_bytes(p.nq, ea, p.rows_m);
    }
    if (p.kind == KIND_COL && p.rows_m == 1) return 0;   // short contraction: b in registers
    if (p.kind == KIND_ROW_PANEL) return 0;               // b in registers, static reduction buffer
    if (p.kind == KIND_ROW_SHIFT) return rs_smem_bytes(p.nq, acc_size(p.dtype), p.dtype == F64 && p.kahan);
    if (p.kind == KIND_ROW)   // fp64 mix: b's split for rows of up to ROW_SPLIT_MAX elements
        return (p.dtype == F64 && p.kahan && p.rows_m == 0 && p.group > 1 && p.nq <= (uint64_t)ROW_SPLIT_MAX)
                   ? ROW_SPLIT_MAX * 8 : 0;
    const size_t es = acc_size(p.dtype);
    const size_t bcap = BSTAGE_BYTES / es + 16 / es;
    // fp64 with the double-float mix: b's split beside the staged b (every column form)
    const size_t split = (p.dtype == F64 && p.kahan) ? bcap * 8 : 0;
    if (p.kind == KIND_COL_THIN) return 16 + bcap * es + split + (size_t)(BLOCK / 32) * 32 * 2 * p.vec * es;
    const size_t WO = (BLOCK / 32) / p.group;
    const size_t red = p.group > 1 ? (size_t)(p.group - 1) * WO * 32 * 2 * p.vec * p.mo * es : 0;
    return 16 + bcap * es + split + red;
}

size_t partial_bytes(const Plan& p)
{
    if (p.split <= 1) return 0;
    return (size_t)p.split * p.S * p.P * 2 * acc_size(p.dtype);
}

// Entry address of a plan's main kernel, for occupancy queries and attributes.
static const void* kernel_entry(const Plan& p)
{
    if (p.kind == KIND_STREAM) return reinterpret_cast<const void*>(stream_fn(p));
    return reinterpret_cast<const void*>(main_kernel(p));
}

int plan_ctas_per_sm(const Plan& p)
{
    static std::mutex mu;
    static std::unordered_map<uint64_t, int> cache;
    const void* fn = kernel_entry(p);
    if (!fn) return 0;
    const size_t smem = plan_smem_bytes(p);
    const uint64_t key = (reinterpret_cast<uintptr_t>(fn) << 20) ^ smem;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    int n = 0;
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int threads = p.kind == KIND_STREAM ? STREAM_THREADS
                        : (p.kind == KIND_ROW_TILE ? ROWT_THREADS : (p.kind == KIND_COL_BULK ? CB_THREADS : BLOCK));
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, threads, smem) !=
        cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = n;
    return n;
}

// One kernel launch, as a programmatic dependent of the stream's previous
// kernel when `dependent` is set (every engine kernel opens with
// pdl_prologue, which waits for that kernel before touching memory).
template <typename... Params, typename... Args>
static cudaError_t launch_ex(void (*fn)(Params...), int grid, int threads, size_t smem, cudaStream_t stream,
                             bool dependent, Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    if (dependent) {
        attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[0].val.programmaticStreamSerializationAllowed = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    return cudaLaunchKernelEx(&cfg, fn, std::forward<Args>(args)...);
}

cudaError_t launch_plan(const Plan& plan, const void* a, const void* b, void* c, void* partial,
                        cudaStream_t stream, uint64_t* launches, bool dependent)
{
    if (plan.kind == KIND_STREAM) {
        SArgs sa;
        sa.a = a;
        sa.b = b;
        sa.out = c;
        sa.partial = partial;
        sa.S = plan.S;
        sa.nq = plan.nq;
        sa.P = plan.P;
        sa.L = plan.L;
        sa.R = plan.R;
        sa.units = plan.units;
        sa.units_per_cta = plan.units_per_cta;
        sa.seg_len = plan.seg_len;
        sa.nseg = (uint32_t)plan.split;
        sa.G = (uint32_t)plan.group;
        sa.RG = (uint32_t)plan.RG;
        sa.J = (uint32_t)plan.J;
        const size_t smem = plan_smem_bytes(plan);
        StreamFn sf = stream_fn(plan);
        if (smem > 48 * 1024)
            cudaFuncSetAttribute(reinterpret_cast<const void*>(sf), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
        cudaError_t err = launch_ex(sf, plan.grid, STREAM_THREADS, smem, stream, dependent, sa);
        if (err != cudaSuccess) return err;
        if (launches) ++*launches;
        if (plan.split > 1) return launch_combine(plan, partial, c, stream, launches);
        return cudaSuccess;
    }
    KernelFn fn = main_kernel(plan);
    if (!fn) return cudaErrorInvalidConfiguration;
    KArgs k;
    k.a = a;
    k.b = b;
    k.out = c;
    k.partial = partial;
    k.S = plan.S;
    k.nq = plan.nq;
    k.P = plan.P;
    k.seg_len = plan.seg_len;
    k.items = plan.items;
    k.items_per_cta = plan.items_per_cta;
    k.nseg = (uint32_t)plan.split;
    k.group = (uint32_t)plan.group;
    if (plan.kind == KIND_COL_THIN) {
        k.ntiles = plan.S;
    } else if (plan.kind == KIND_COL_BULK) {
        k.ntiles = (plan.P + col_bulk_tile(plan.dtype) - 1) / col_bulk_tile(plan.dtype);   // tiles per slice
    } else if (plan.kind == KIND_ROW_PANEL) {
        k.ntiles = (plan.S + plan.items_per_cta - 1) / plan.items_per_cta;   // row blocks per segment
    } else if (plan.kind == KIND_COL && plan.rows_m == 1) {
        k.ntiles = 0;   // pairs of tiles of BLOCK * V outputs are the items
    } else if (plan.kind == KIND_COL || plan.kind == KIND_COL_REALIGN) {
        const uint64_t TO = uint64_t((BLOCK / 32) / plan.group) * 32u * plan.vec * plan.mo;
        k.ntiles = (plan.S * plan.P + TO - 1) / TO;
    } else {
        k.ntiles = 0;
    }
    if (plan.kind == KIND_COL_BULK) {
        // item -> segment (S * ntiles items each), then -> slice (ntiles each)
        k.tdiv = make_idx_div(plan.S * k.ntiles, plan.items);
        k.pdiv = make_idx_div(k.ntiles, plan.S * k.ntiles);
    } else {
        k.pdiv = make_idx_div(plan.P, plan.S * plan.P);
        k.tdiv = make_idx_div(k.ntiles, plan.items);
    }
    const size_t smem = plan_smem_bytes(plan);
    if ((plan.kind == KIND_ROW_TILE || plan.kind == KIND_COL_BULK) && smem > 48 * 1024)
        cudaFuncSetAttribute(reinterpret_cast<const void*>(fn), cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int threads = plan.kind == KIND_ROW_TILE ? ROWT_THREADS : (plan.kind == KIND_COL_BULK ? CB_THREADS : BLOCK);
    cudaError_t err = launch_ex(fn, plan.grid, threads, smem, stream, dependent, k);
    if (err != cudaSuccess) return err;
    if (launches) ++*launches;
    if (plan.split > 1) return launch_combine(plan, partial, c, stream, launches);
    return cudaSuccess;
}

cudaError_t launch_combine(const Plan& plan, void* partial, void* c, cudaStream_t stream, uint64_t* launches)
{
    cudaError_t err;
    {
        const uint64_t outputs = plan.S * plan.P;
        const uint64_t sms = plan.sms > 0 ? (uint64_t)plan.sms : (uint64_t)PLAN_SMS_WITHOUT_DEVICE;
        // threads per output: one when the outputs alone fill the GPU, else enough
        // to give each thread about eight segments
        uint32_t tpo = 1;
        if (outputs < sms * BLOCK * 4 && plan.split >= 16) {
            tpo = 1;
            while (tpo * 2 <= (uint32_t)BLOCK && tpo * 2 * 8 <= (uint32_t)plan.split) tpo *= 2;
        }
        const uint64_t opb = BLOCK / tpo;
        int g = (int)std::min<uint64_t>(sms * 16, (outputs + opb - 1) / opb);
        if (g < 1) g = 1;
        const uint32_t ns = (uint32_t)plan.split;
        switch (plan.dtype) {
        case F32:
        case BF16A: {
            const Pair<float>* pf = static_cast<const Pair<float>*>(partial);
            float* cf = static_cast<float*>(c);
            if (plan.f64_combine)
                err = launch_ex(combine_kernel<float, true, true>, g, BLOCK, 0, stream, true, pf, cf, outputs, ns, tpo);
            else if (plan.kahan)
                err = launch_ex(combine_kernel<float, true, false>, g, BLOCK, 0, stream, true, pf, cf, outputs, ns, tpo);
            else
                err = launch_ex(combine_kernel<float, false, false>, g, BLOCK, 0, stream, true, pf, cf, outputs, ns,
                                tpo);
            break;
        }
        case F64:
            err = launch_ex(combine_kernel<double, false, false>, g, BLOCK, 0, stream, true,
                            static_cast<const Pair<double>*>(partial), static_cast<double*>(c), outputs, ns, tpo);
            break;
        default:
            err = cudaErrorInvalidValue;
        }
        if (err != cudaSuccess) return err;
        if (launches) ++*launches;
    }
    return cudaSuccess;
}

// Self-test of the expiry path: an mbarrier nothing arrives at, waited on
// with a short poll limit; the wait gives up, sets the device error word and
// the kernel returns (no trap, no fault, the context stays usable).
__global__ void wait_expiry_probe(uint32_t limit)
{
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait_bounded(&bar, 0u, &g_device_error, limit);
}

cudaError_t launch_wait_probe(cudaStream_t stream, uint32_t limit)
{
    wait_expiry_probe<<<1, 32, 0, stream>>>(limit);
    return cudaGetLastError();
}

unsigned int read_and_clear_device_error()
{
    unsigned int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_device_error, sizeof(v)) != cudaSuccess) return 0xffffffffu;
    cudaMemcpyToSymbol(g_device_error, &zero, sizeof(zero));
    return v;
}

}  // namespace tlibg
