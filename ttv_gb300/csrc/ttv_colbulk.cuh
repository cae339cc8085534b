// Column kernel with TMA-staged rows (included by ttv_kernels.cu, after
// ttv_stream.cuh).
//
// A work item is (segment of q, slice s, tile of CB_TJ = 4 KB of consecutive
// outputs of the prefix); its rows i are the runs A[s, i, j0 .. j0 + TJ).
// The last warp is the producer: for each block of CB_RB rows of the CTA's
// walk it waits until the consumers have released the stage (empty mbarrier),
// writes b[i] of the block's rows (and, for fp64, their double-float split)
// into the stage, and issues one 1-D bulk copy (cp.async.bulk) per row of the
// 16-byte-aligned cover of the row's run (at most 15 bytes on either side,
// inside the same 16-byte chunks as the run's first and last element, so
// inside the allocation) against the stage's full mbarrier.  The CB_CONSUMERS
// threads before it wait on the full barrier, read their elements of each row
// from shared memory at the row's own misalignment, accumulate, and release
// the stage.  The ring of CB_NS stages, not registers, holds the bytes in
// flight.  Thread t owns the outputs j0 + t + CB_CONSUMERS v (v < V): each
// shared-memory read of a warp is 32 consecutive elements and each store of C
// is coalesced.  Every wait is
// bounded; on expiry the CTA records the device error, waits (bounded) for its
// own copies in flight and leaves.
#pragma once

namespace tlibg {

template <typename TA> __host__ __device__ constexpr int cb_tj() { return CB_ROW_BYTES / (int)sizeof(TA); }
// stage layout: CB_RB row slots, then b of those rows (8 bytes each), their
// split (float2) and their in-window flags
constexpr int CB_STAGE = CB_RB * CB_ROWB + CB_RB * 8 + CB_RB * 8 + CB_RB * 4;
constexpr int CB_STAGE_AL = (CB_STAGE + 127) / 128 * 128;

// The CTA's walk over (item, row block) pairs, identical for producer and consumers.
struct CbWalk {
    uint64_t item, last;   // current item, end of the CTA's items
    uint64_t seg, s, tile;
    uint64_t i0, ie;       // current block's first row, the item's row end
    __device__ __forceinline__ void set_item(const KArgs& k)
    {
        if (item >= last) return;
        seg = idx_div(item, k.tdiv);                   // items per segment: S * ntiles
        const uint64_t rest = item - seg * (k.S * k.ntiles);
        s = idx_div(rest, k.pdiv);                     // tiles per slice
        tile = rest - s * k.ntiles;
        i0 = seg * k.seg_len;
        ie = min(k.nq, i0 + k.seg_len);
    }
    __device__ __forceinline__ void begin(const KArgs& k)
    {
        item = (uint64_t)blockIdx.x * k.items_per_cta;
        last = min(k.items, item + k.items_per_cta);
        set_item(k);
    }
    __device__ __forceinline__ bool valid() const { return item < last; }
    __device__ __forceinline__ uint32_t rows() const { return (uint32_t)min((uint64_t)CB_RB, ie - i0); }
    __device__ __forceinline__ bool last_block() const { return i0 + CB_RB >= ie; }
    __device__ __forceinline__ void next(const KArgs& k)
    {
        if (last_block()) {
            ++item;
            set_item(k);
        } else {
            i0 += CB_RB;
        }
    }
};

// Producer warp: b (and its split) of the walk's current block into the stage,
// then one bulk copy per row.
template <typename TA, typename T, bool PRES>
__device__ __forceinline__ void cb_produce(const KArgs& k, const CbWalk& w, unsigned char* st, uint64_t* full,
                                           uint32_t lane)
{
    constexpr int TJ = cb_tj<TA>();
    const TA* A = static_cast<const TA*>(k.a);
    const T* B = static_cast<const T*>(k.b);
    const uint32_t nr = w.rows();
    T* sbv = reinterpret_cast<T*>(st + CB_RB * CB_ROWB);
    float2* ssp = reinterpret_cast<float2*>(st + CB_RB * CB_ROWB + CB_RB * 8);
    int* sok = reinterpret_cast<int*>(st + CB_RB * CB_ROWB + CB_RB * 16);
    if (lane < nr) {
        const T bb = __ldg(B + w.i0 + lane);
        sbv[lane] = bb;
        if constexpr (PRES) {
            const DSplit d = split_double(bb);
            ssp[lane] = make_float2(d.hi, d.lo);
            sok[lane] = d.ok ? 1 : 0;
        }
    }
    __syncwarp();
    if (lane == 0) {
        const uint64_t j0 = w.tile * TJ;
        const uint64_t ncols = min((uint64_t)TJ, k.P - j0);
        uint32_t total = 0;
        const uintptr_t g00 = reinterpret_cast<uintptr_t>(A + ((w.s * k.nq + w.i0) * k.P + j0));
        const uintptr_t rowb = k.P * sizeof(TA);
        for (uint32_t r = 0; r < nr; ++r) {
            const uintptr_t g0 = g00 + r * rowb;
            total += (uint32_t)(((g0 + ncols * sizeof(TA) + 15) & ~uintptr_t(15)) - (g0 & ~uintptr_t(15)));
        }
        fence_proxy_async_smem();   // the stage's earlier generic reads before the async writes
        mbar_arrive_expect_tx(full, total);
        for (uint32_t r = 0; r < nr; ++r) {
            const uintptr_t g0 = g00 + r * rowb;
            const uintptr_t c0 = g0 & ~uintptr_t(15);
            const uint32_t bytes = (uint32_t)(((g0 + ncols * sizeof(TA) + 15) & ~uintptr_t(15)) - c0);
            bulk_g2s(st + (size_t)r * CB_ROWB, reinterpret_cast<const void*>(c0), bytes, full);
        }
    }
}

template <typename TA, typename T, bool KAHAN>
__global__ void __launch_bounds__(CB_THREADS) col_bulk_kernel(KArgs k)
{
    pdl_prologue();
    constexpr int TJ = cb_tj<TA>();
    constexpr int V = TJ / CB_CONSUMERS;
    constexpr bool PRES = presplit_b<T, KAHAN>();
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
    uint64_t* empty = full + CB_NS;
    unsigned char* ring = smem_raw + 128;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const TA* __restrict__ A = static_cast<const TA*>(k.a);

    if (threadIdx.x == 0) {
        for (int s = 0; s < CB_NS; ++s) {
            mbar_init(full + s, 1);
            mbar_init(empty + s, CB_CONSUMERS / 32);
        }
        fence_mbar_init();
    }
    __syncthreads();

    CbWalk w;
    w.begin(k);
    if (warp == CB_CONSUMERS / 32) {
        // ---------------- producer ----------------
        uint64_t g = 0;
        for (; w.valid(); ++g) {
            const uint32_t slot = (uint32_t)(g % CB_NS);
            if (g >= (uint64_t)CB_NS) {
                const bool ok = mbar_wait_bounded(empty + slot, (uint32_t)(((g / CB_NS) - 1) & 1), &g_device_error);
                if (__any_sync(0xffffffffu, !ok)) break;
            }
            cb_produce<TA, T, PRES>(k, w, ring + (size_t)slot * CB_STAGE_AL, full + slot, lane);
            w.next(k);
        }
        // the latest phase of every stage used: its copies have landed before the CTA retires
        if (lane == 0)
            for (uint64_t h = (g > (uint64_t)CB_NS ? g - CB_NS : 0); h < g; ++h)
                mbar_wait_bounded(full + (h % CB_NS), (uint32_t)((h / CB_NS) & 1), &g_device_error);
        return;
    }

    // ---------------- consumers ----------------
    const uint32_t t = threadIdx.x;
    typename AccSel<T, KAHAN>::type acc[V];
#pragma unroll
    for (int v = 0; v < V; ++v) acc[v].init();
    for (uint64_t g = 0; w.valid(); ++g) {
        const uint32_t slot = (uint32_t)(g % CB_NS);
        const bool ok = mbar_wait_bounded(full + slot, (uint32_t)((g / CB_NS) & 1), &g_device_error);
        if (__any_sync(0xffffffffu, !ok)) return;
        const unsigned char* st = ring + (size_t)slot * CB_STAGE_AL;
        const T* sbv = reinterpret_cast<const T*>(st + CB_RB * CB_ROWB);
        const float2* ssp = reinterpret_cast<const float2*>(st + CB_RB * CB_ROWB + CB_RB * 8);
        const int* sok = reinterpret_cast<const int*>(st + CB_RB * CB_ROWB + CB_RB * 16);
        const uint64_t j0 = w.tile * TJ;
        const uint32_t ncols = (uint32_t)min((uint64_t)TJ, k.P - j0);
        const uint32_t nr = w.rows();
        // misalignment of the block's first row; rows advance by P elements
        uint32_t mis = (uint32_t)(reinterpret_cast<uintptr_t>(A + ((w.s * k.nq + w.i0) * k.P + j0)) & 15u);
        const uint32_t step = (uint32_t)((k.P * sizeof(TA)) & 15u);
        const bool full_tile = ncols == (uint32_t)TJ;
#pragma unroll
        for (int r = 0; r < CB_RB; ++r) {
            if ((uint32_t)r < nr) {
                const TA* row = reinterpret_cast<const TA*>(st + (size_t)r * CB_ROWB + mis);
                T av[V];
#pragma unroll
                for (int v = 0; v < V; ++v)
                    av[v] = (full_tile || t + CB_CONSUMERS * v < ncols) ? Cvt<TA, T>::f(row[t + CB_CONSUMERS * v])
                                                                       : T(0);
                if constexpr (PRES) {
                    if (sok[r])
                        row_fma<V, true>(acc, av, sbv[r], r, ssp + r);
                    else
                        row_fma<V, false>(acc, av, sbv[r], r, nullptr);
                } else {
                    row_fma<V, false>(acc, av, sbv[r], r, nullptr);
                }
                mis = (mis + step) & 15u;
            }
        }
        renorm_all<V>(acc);
        __syncwarp();
        if (lane == 0) mbar_arrive(empty + slot);   // this warp is done with the stage
        if (w.last_block()) {
#pragma unroll
            for (int v = 0; v < V; ++v) acc[v].fold();
            const uint64_t outputs = k.S * k.P;
#pragma unroll
            for (int v = 0; v < V; ++v) {
                const uint32_t jj = t + CB_CONSUMERS * v;
                if (jj < ncols) {
                    const uint64_t o = w.s * k.P + j0 + jj;
                    if (k.nseg == 1) {
                        static_cast<T*>(k.out)[o] = acc[v].value();
                    } else {
                        Pair<T> pr;
                        pr.s = acc[v].s;
                        pr.c = KAHAN ? acc[v].c : T(0);
                        static_cast<Pair<T>*>(k.partial)[w.seg * outputs + o] = pr;
                    }
                }
                acc[v].init();
            }
        }
        w.next(k);
    }
}

}  // namespace tlibg
