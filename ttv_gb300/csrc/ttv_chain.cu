// Fused multi-vector chain: C = A x_1 b_1 ... (every mode but q) ... x_p b_p.
//
// The reference's ttvpy.ttvs (ttvpy/src/wrapped_ttv.cpp:85-199) runs p - 1
// separate TTVs, each reading the previous intermediate and allocating the
// next.  Here the chain reads A once.  In the canonical view of A with
// respect to q, A = (S, n_q, P) row-major (P: the extents laid out before q,
// S: those after), the result is
//
//     c[i] = sum_s wS[s] * sum_j A[s, i, j] * wP[j],
//
// where wP and wS are the Kronecker products of the vectors of the prefix and
// suffix modes (in layout order).  So the chain is
//   1. kron_kernel      wP and wS from the p - 1 vectors (products in fp64,
//                       rounded once to the element type)
//   2. row TTV          D[s, i] = sum_j A[s, i, j] wP[j]: rows of the
//                       contiguous prefix (the engine's row-form kernels;
//                       skipped when P == 1)
//   3. column TTV       c[i] = sum_s wS[s] D[s, i] (the column-form kernels;
//                       skipped when S == 1)
// with no host synchronisation and no allocation after the first call on a
// stream (wP, wS, D and split partials live in the stream's cached scratch).
// Every contraction order of the reference gives the same sum up to
// rounding; this one reads A once whatever order is asked for.
#include "ttv_internal.h"

#include <string>
#include <vector>

namespace tlibg {

constexpr int KRON_MAX_MODES = 32;

struct KronArgs {
    const void* vec[KRON_MAX_MODES];   // prefix modes first (layout order), then suffix modes
    uint64_t ext[KRON_MAX_MODES];
    int np, ns;                        // number of prefix / suffix modes
    uint64_t P, S;
    void* wP;
    void* wS;
};

// One weight per thread: the mixed-radix digits of its index pick one element
// of each mode's vector.  I: 32-bit index arithmetic when P + S < 2^32 (one
// 32-bit division per mode instead of a 64-bit one).
template <typename T, typename I>
__global__ void kron_kernel(KronArgs k)
{
    const I P = (I)k.P, total = (I)(k.P + k.S);
    for (I idx = (I)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (I)gridDim.x * blockDim.x) {
        const bool pre = idx < P;
        I j = pre ? idx : idx - P;
        const int m0 = pre ? 0 : k.np, m1 = pre ? k.np : k.np + k.ns;
        double w = 1.0;
        for (int m = m0; m < m1; ++m) {
            const I e = (I)k.ext[m];
            const I q = j / e;
            w *= (double)static_cast<const T*>(k.vec[m])[j - q * e];
            j = q;
        }
        if (pre)
            static_cast<T*>(k.wP)[idx] = (T)w;
        else
            static_cast<T*>(k.wS)[idx - P] = (T)w;
    }
}

namespace {

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

const char* const E_ORDER = "Error calling ttvpy::ttvs: input tensor order should be greater than zero.";
const char* const E_MODE =
    "Error calling ttvpy::ttvs: contraction mode should be greater than zero or less than or equal to p.";
const char* const E_DIM =
    "Error calling ttvpy::ttvs: vector dimension is not compatible with the dimension of a tensor mode.";

}  // namespace
}  // namespace tlibg

using namespace tlibg;

extern "C" int tlibg_ttvs(int dtype, size_t q, size_t p, const void* a, const size_t* na, const size_t* wa,
                          const size_t* pia, const void* const* bs, const size_t* nbs, void* c, void* stream)
{
    NvtxRange nvtx("tlibg_ttvs");
    if (dtype != F32 && dtype != F64 && dtype != BF16A) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg: unknown element type");
    if (p == 0) return internal_fail(TLIBG_ERR_ARGUMENT, E_ORDER);
    if (q == 0 || q > p) return internal_fail(TLIBG_ERR_ARGUMENT, E_MODE);
    if (!a || !c || !na || !wa || !pia || (p > 1 && (!bs || !nbs)))
        return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_ttvs: null pointer argument");
    if (p == 1)
        return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_ttvs: a tensor of order 1 has no mode to contract "
                                                 "besides q");
    if (p > (size_t)KRON_MAX_MODES + 1)
        return internal_fail(TLIBG_ERR_UNSUPPORTED, "tlibg_ttvs: at most 33 modes");
    // vectors in mode order, skipping q: bs[r] belongs to mode r + 1 (r < q - 1) or r + 2
    for (size_t r = 0; r + 1 < p; ++r) {
        const size_t mode = r + 1 < q ? r + 1 : r + 2;
        if (nbs[r] != na[mode - 1]) return internal_fail(TLIBG_ERR_ARGUMENT, E_DIM);
        if (!bs[r]) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_ttvs: null vector pointer");
    }
    // A through the validation of the single call: a TTV over mode q with b = bs[0]
    // stands in for the metadata checks (shape, layout, dense strides)
    std::vector<size_t> nc(p - 1), pic(p - 1), wc(p - 1);
    if (int st = tlibg_output_shape(na, p, q, nc.data())) return st;
    if (int st = tlibg_output_layout(pia, p, q, pic.data())) return st;
    if (int st = tlibg_strides(nc.data(), pic.data(), p - 1, wc.data())) return st;
    CanonView cn;
    const size_t nbq = na[q - 1];
    if (int st = internal_analyse(q, p, a, na, wa, pia, bs[0], &nbq, c, nc.data(), wc.data(), pic.data(), &cn))
        return st;
    const size_t ea = dtype == F64 ? 8 : (dtype == BF16A ? 2 : 4), et = dtype == F64 ? 8 : 4;
    const int tdt = dtype == F64 ? F64 : F32;   // type of b, the weights, D and c
    if ((reinterpret_cast<uintptr_t>(a) % ea) || (reinterpret_cast<uintptr_t>(c) % et))
        return internal_fail(TLIBG_ERR_UNSUPPORTED, "tlibg: a, b and c must be aligned to their element sizes");
    for (size_t r = 0; r + 1 < p; ++r)
        if (reinterpret_cast<uintptr_t>(bs[r]) % et)
            return internal_fail(TLIBG_ERR_UNSUPPORTED, "tlibg: a, b and c must be aligned to their element sizes");
    const int sms = internal_sms();
    if (!sms) return internal_fail(TLIBG_ERR_CUDA, "tlibg: no usable CUDA device");
    if (int st = internal_check_device_pointers(a, c, c)) return st;
    for (size_t r = 0; r + 1 < p; ++r)
        if (int st = internal_check_device_pointers(bs[r], bs[r], bs[r])) return st;

    // Kronecker factors: prefix modes in layout order (fastest first), then suffix modes
    KronArgs ka{};
    size_t k = 0;
    while (pia[k] != q) ++k;
    auto vec_of = [&](size_t mode) { return bs[mode < q ? mode - 1 : mode - 2]; };
    int nm = 0;
    for (size_t r = 0; r < k; ++r) {
        ka.vec[nm] = vec_of(pia[r]);
        ka.ext[nm++] = na[pia[r] - 1];
    }
    ka.np = nm;
    for (size_t r = k + 1; r < p; ++r) {
        ka.vec[nm] = vec_of(pia[r]);
        ka.ext[nm++] = na[pia[r] - 1];
    }
    ka.ns = nm - ka.np;
    ka.P = cn.P;
    ka.S = cn.S;
    const uint64_t P = cn.P, S = cn.S, nq = cn.nq;
    const bool stage1 = P > 1, stage2 = S > 1;

    // plans (pointers for the alignment rules: scratch regions are 256-byte aligned)
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const size_t off_wP = 0;
    const size_t off_wS = off_wP + align256(stage1 ? P * et : 0);
    const size_t off_D = off_wS + align256(stage2 ? S * et : 0);
    const size_t off_part = off_D + align256(stage1 && stage2 ? S * nq * et : 0);
    static const uint4 probe[1] = {};   // 256-byte aligned stand-in for scratch regions
    Plan pl1, pl2;
    if (stage1) {
        CanonView c1;
        c1.P = 1;
        c1.nq = P;
        c1.S = S * nq;
        if (int s = internal_plan(dtype, c1, a, probe, nullptr, sms, &pl1)) return s;
    }
    if (stage2) {
        CanonView c2;
        c2.P = nq;
        c2.nq = S;
        c2.S = 1;
        if (int s = internal_plan(stage1 ? tdt : dtype, c2, stage1 ? (const void*)probe : a, probe, nullptr, sms, &pl2))
            return s;
    }
    const size_t part_bytes = std::max(stage1 ? partial_bytes(pl1) : 0, stage2 ? partial_bytes(pl2) : 0);
    void* scratch = nullptr;
    if (int s = internal_scratch(st, off_part + part_bytes, &scratch)) return s;
    char* base = static_cast<char*>(scratch);
    void* wP = base + off_wP;
    void* wS = base + off_wS;
    void* D = stage1 && stage2 ? base + off_D : c;
    void* part = base + off_part;
    ka.wP = wP;
    ka.wS = wS;

    uint64_t launches = 0;
    const uint64_t nk = (stage1 ? P : 0) + (stage2 ? S : 0);
    if (!stage1) ka.P = 0;
    if (!stage2) ka.S = 0;
    if (nk) {
        const int grid = (int)std::min<uint64_t>((uint64_t)sms * 8, (nk + 255) / 256);
        const bool narrow = nk < (uint64_t(1) << 32);
        if (tdt == F64) {
            if (narrow) kron_kernel<double, uint32_t><<<grid, 256, 0, st>>>(ka);
            else kron_kernel<double, uint64_t><<<grid, 256, 0, st>>>(ka);
        } else {
            if (narrow) kron_kernel<float, uint32_t><<<grid, 256, 0, st>>>(ka);
            else kron_kernel<float, uint64_t><<<grid, 256, 0, st>>>(ka);
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return internal_cuda_fail(e, "kernel launch");
        ++launches;
    }
    if (stage1) {
        cudaError_t e = launch_plan(pl1, a, wP, D, part, st, &launches);
        if (e != cudaSuccess) return internal_cuda_fail(e, "kernel launch");
    }
    if (stage2) {
        cudaError_t e = launch_plan(pl2, stage1 ? D : a, wS, c, part, st, &launches);
        if (e != cudaSuccess) return internal_cuda_fail(e, "kernel launch");
    }
    internal_count_launches(launches);
    return internal_ok();
}
