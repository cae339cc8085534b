// Fused multi-vector chain: C = A x_1 b_1 ... (every mode but q) ... x_p b_p.
//
// The reference's ttvpy.ttvs (ttvpy/src/wrapped_ttv.cpp:85-199) runs p - 1
// separate TTVs, each reading the previous intermediate and allocating the
// next.  Here the chain reads A once, in a short sequence of stages planned
// on the host.  Walk the modes of A in layout order (fastest first); q sits
// at position k.  A stage contracts a contiguous group of modes at one end
// of the layout:
//   * first stage, row form (k > 0): the fastest mode alone when it is long
//     and its rows are whole 16-byte vectors, else the fastest modes as few as
//     make rows of at least CHAIN_MIN_ROW elements (or all modes before q);
//   * first stage, column form (q fastest): the slowest modes, as many as
//     leave at least CHAIN_MIN_OUTPUTS outputs (at least one mode);
//   * later stages: all remaining modes on one side of q (a column stage over
//     a large intermediate keeps CHAIN_LATE_OUTPUTS outputs).
// Each stage runs on the engine's own planner and kernels.  A stage over one
// mode reads that mode's vector in place; stages over several modes read the
// Kronecker product of their vectors (computed in fp64, rounded once to the
// element type), all built by one kernel launch.  The first stage reads A
// (about all the traffic); each later one reads the previous, much smaller,
// intermediate.  Intermediates live in the stream's cached scratch: no host
// synchronisation and no allocation after the first call on a stream.  Each
// launch after the first is a programmatic dependent of the one before, so
// its launch overlaps its predecessor's tail.
// Every contraction order of the reference gives the same sum up to
// rounding; this one reads A once whatever order is asked for.
#include "ttv_internal.h"

#include <string>
#include <vector>

namespace tlibg {

constexpr int KRON_MAX_MODES = 32;
constexpr int KRON_MAX_GROUPS = KRON_MAX_MODES;   // one weight vector per stage
#ifndef TLIBG_CHAIN_MIN_ROW
#define TLIBG_CHAIN_MIN_ROW 2048
#endif
#ifndef TLIBG_CHAIN_MIN_OUTPUTS
#define TLIBG_CHAIN_MIN_OUTPUTS 65536
#endif
constexpr uint64_t CHAIN_MIN_ROW = TLIBG_CHAIN_MIN_ROW;           // row stage: rows at least this long
constexpr uint64_t CHAIN_MIN_OUTPUTS = TLIBG_CHAIN_MIN_OUTPUTS;   // column stage: at least this many outputs
constexpr uint64_t CHAIN_ONE_MODE_ROW = 64;           // first row stage: one mode if it is this long
#ifndef TLIBG_CHAIN_SEG_KB
#define TLIBG_CHAIN_SEG_KB 128
#endif
#ifndef TLIBG_CHAIN_SPLIT_CAP
#define TLIBG_CHAIN_SPLIT_CAP 1
#endif
constexpr uint64_t CHAIN_SEG_BYTES = (uint64_t)TLIBG_CHAIN_SEG_KB << 10;   // later stages: bytes per split segment
constexpr uint64_t CHAIN_SMALL = uint64_t(1) << 22;   // intermediates up to this many elements: one stage
constexpr uint64_t CHAIN_LATE_OUTPUTS = 4096;         // larger ones: column stages keep this many outputs

// Weight vectors of the stages: group g has modes [m0[g], m1[g]) of vec/ext
// (fastest first, each new mode slower) and writes len[g] weights at
// out + off[g] (elements; every group starts 256-byte aligned).
struct KronArgs {
    const void* vec[KRON_MAX_MODES];
    uint64_t ext[KRON_MAX_MODES];
    int m0[KRON_MAX_GROUPS], m1[KRON_MAX_GROUPS];
    uint64_t off[KRON_MAX_GROUPS + 1];   // group starts; off[ngroups] = end of the last
    uint64_t len[KRON_MAX_GROUPS];
    int ngroups;
    void* out;
};

// One weight per thread: the mixed-radix digits of its index within its group
// pick one element of each of the group's vectors.  I: 32-bit index
// arithmetic when the weights number fewer than 2^32.
template <typename T, typename I, bool AFTER>
__global__ void kron_kernel(KronArgs k)
{
    // AFTER: launched as a programmatic dependent of the first stage, which does not
    // read the weights: let the next stage be scheduled, compute, and only then wait
    // for the first stage, so that a kernel waiting for this one also waits for it.
    // Otherwise the engine kernels' usual prologue (wait, then allow dependents; the
    // wait returns at once when launched normally).
    if (AFTER)
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    else
        asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory");
    const I total = (I)k.off[k.ngroups];
    for (I idx = (I)blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += (I)gridDim.x * blockDim.x) {
        int g = 0;
        while ((I)k.off[g + 1] <= idx) ++g;
        I j = idx - (I)k.off[g];
        if (j >= (I)k.len[g]) continue;   // alignment gap after the group
        double w = 1.0;
        for (int m = k.m0[g]; m < k.m1[g]; ++m) {
            const I e = (I)k.ext[m];
            const I q = j / e;
            w *= (double)static_cast<const T*>(k.vec[m])[j - q * e];
            j = q;
        }
        static_cast<T*>(k.out)[idx] = (T)w;
    }
    if (AFTER) asm volatile("griddepcontrol.wait;" ::: "memory");
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

    // modes in layout order, fastest first: extent and vector (q: none)
    std::vector<uint64_t> ext;
    std::vector<const void*> vec;
    for (size_t r = 0; r < p; ++r) {
        const size_t m = pia[r];
        ext.push_back(na[m - 1]);
        vec.push_back(m == q ? nullptr : bs[m < q ? m - 1 : m - 2]);
    }
    size_t kq = 0;
    while (pia[kq] != q) ++kq;

    // stages: [lo, hi) modes of the current tensor contracted, row or column form
    struct Stage {
        bool row;
        int group;         // weight group of the Kronecker launch, or -1: one mode, its vector
        const void* w;     // the vector (group < 0)
        uint64_t L, R;     // row: rows R of length L; column: outputs L, contracted rows R
    };
    std::vector<Stage> stages;
    KronArgs ka{};
    int nv = 0;
    uint64_t wtot = 0, N = 1;
    for (uint64_t e : ext) N *= e;
    {
        std::vector<uint64_t> ex = ext;
        std::vector<const void*> ve = vec;
        size_t k = kq;
        uint64_t n = N;
        while (ex.size() > 1) {
            // The first stage reads A: rows long enough (row form) or outputs enough
            // (column form) for the engine's kernels to stream at full rate.  Later
            // stages read an intermediate that is orders of magnitude smaller: each
            // takes all remaining modes on its side of q (a column stage over an
            // intermediate of more than CHAIN_SMALL elements stops at
            // CHAIN_LATE_OUTPUTS outputs), so one to three follow.
            const bool first = stages.empty();
            Stage sg{};
            size_t lo, hi;
            if (k > 0) {
                // rows of the fastest mode alone when they are long and whole 16-byte
                // vectors: that stage needs no Kronecker weights, so the weight launch
                // for the later stages overlaps it
                const bool one = first && ex[0] >= CHAIN_ONE_MODE_ROW && (ex[0] * ea) % 16 == 0;
                uint64_t L = 1;
                hi = 0;
                while (hi < k && (!first || hi == 0 || (!one && L < CHAIN_MIN_ROW))) L *= ex[hi++];
                lo = 0;
                sg.row = true;
                sg.L = L;
                sg.R = n / L;
            } else {
                // a large intermediate keeps enough outputs for the column kernels too
                // (a GEMV with a few dozen outputs over megabytes is latency-bound)
                const uint64_t min_out = first ? CHAIN_MIN_OUTPUTS : (n > CHAIN_SMALL ? CHAIN_LATE_OUTPUTS : 0);
                uint64_t inner = ex[0];
                lo = 1;
                while (lo + 1 < ex.size() && inner < min_out) inner *= ex[lo++];
                hi = ex.size();
                sg.row = false;
                sg.L = inner;
                sg.R = n / inner;
            }
            if (hi - lo == 1) {
                sg.group = -1;
                sg.w = ve[lo];
            } else {
                const int g = ka.ngroups++;
                sg.group = g;
                ka.m0[g] = nv;
                for (size_t r = lo; r < hi; ++r) {
                    ka.vec[nv] = ve[r];
                    ka.ext[nv++] = ex[r];
                }
                ka.m1[g] = nv;
                const uint64_t wl = sg.row ? sg.L : sg.R;
                ka.off[g] = wtot;
                ka.len[g] = wl;
                wtot += align256(wl * et) / et;
            }
            stages.push_back(sg);
            // the intermediate keeps the other modes, in the same order
            ex.erase(ex.begin() + lo, ex.begin() + hi);
            ve.erase(ve.begin() + lo, ve.begin() + hi);
            if (sg.row) k -= hi;
            n = sg.row ? sg.R : sg.L;
        }
    }
    ka.off[ka.ngroups] = wtot;

    // plans and scratch: weights, two intermediates, split partials
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    static const uint4 probe[1] = {};   // aligned stand-in for scratch regions
    std::vector<Plan> plans(stages.size());
    size_t part_bytes = 0, inter = 0;
    for (size_t i = 0; i < stages.size(); ++i) {
        const Stage& sg = stages[i];
        CanonView cv;
        if (sg.row) {
            cv.P = 1;
            cv.nq = sg.L;
            cv.S = sg.R;
        } else {
            cv.P = sg.L;
            cv.nq = sg.R;
            cv.S = 1;
        }
        const int dt = i == 0 ? dtype : tdt;
        const void* pw = sg.group < 0 ? sg.w : (const void*)probe;
        if (int s = internal_plan(dt, cv, i == 0 ? a : (const void*)probe, pw, nullptr, sms, &plans[i])) return s;
        if (i > 0 && TLIBG_CHAIN_SPLIT_CAP && plans[i].kind == KIND_COL_THIN) {
            // A later stage reads an intermediate that the stage before has just
            // written (in L2 when small): the thin-prefix kernel's split, sized to fill
            // the GPU twice over HBM-resident data, leaves thousands of partials to
            // combine.  Segments of CHAIN_SEG_BYTES (and at most 256 rows, and at
            // least half as many segments as SMs) are enough here (128^4 fp32, q = 3
            // and 4: 2-3 us less per call; other kernels measured no gain).
            const uint64_t want = std::max(std::max<uint64_t>(cv.P * cv.nq * cv.S * et / CHAIN_SEG_BYTES, cv.nq / 256),
                                           std::max<uint64_t>((uint64_t)sms / 2, 1));
            if (plans[i].split > 1 && (uint64_t)plans[i].split > want) {
                tlibg_options o{TLIBG_ACC_COMPENSATED, -1, 0, 0, (int)want, 0};
                Plan alt;
                if (internal_plan(dt, cv, probe, pw, &o, sms, &alt) == 0) plans[i] = alt;
            }
        }
        part_bytes = std::max(part_bytes, partial_bytes(plans[i]));
        if (i + 1 < stages.size()) inter = std::max<size_t>(inter, (size_t)(sg.row ? sg.R : sg.L));
    }
    const size_t off_w = 0;
    const size_t off_d0 = off_w + align256(wtot * et);
    const size_t off_d1 = off_d0 + align256(inter * et);
    const size_t off_part = off_d1 + align256(stages.size() > 2 ? inter * et : 0);
    void* scratch = nullptr;
    if (int s = internal_scratch(st, off_part + part_bytes, &scratch)) return s;
    char* base = static_cast<char*>(scratch);
    ka.out = base + off_w;

    // The weights: one launch for every group, then the stages, each launched as a
    // programmatic dependent of the kernel before it (it waits for that kernel in
    // its prologue).  When the first stage contracts a single mode it needs no
    // weights: it goes first and the weight launch follows it as a dependent that
    // computes at once, beside the stage, and waits for it only before exiting,
    // so the next stage (waiting for the weights) also comes after the first.
    uint64_t launches = 0;
    const bool weights_after = ka.ngroups > 0 && stages[0].group < 0;
    auto launch_weights = [&](bool dependent) -> cudaError_t {
        const int grid = (int)std::min<uint64_t>((uint64_t)sms * 8, (wtot + 255) / 256);
        const bool narrow = wtot < (uint64_t(1) << 32);
        void (*fn)(KronArgs);
        if (tdt == F64)
            fn = narrow ? (dependent ? kron_kernel<double, uint32_t, true> : kron_kernel<double, uint32_t, false>)
                        : (dependent ? kron_kernel<double, uint64_t, true> : kron_kernel<double, uint64_t, false>);
        else
            fn = narrow ? (dependent ? kron_kernel<float, uint32_t, true> : kron_kernel<float, uint32_t, false>)
                        : (dependent ? kron_kernel<float, uint64_t, true> : kron_kernel<float, uint64_t, false>);
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid);
        cfg.blockDim = dim3(256);
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        if (dependent) {
            attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
            attr[0].val.programmaticStreamSerializationAllowed = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
        }
        cudaError_t e = cudaLaunchKernelEx(&cfg, fn, ka);
        if (e == cudaSuccess) ++launches;
        return e;
    };
    if (ka.ngroups > 0 && !weights_after) {
        cudaError_t e = launch_weights(false);
        if (e != cudaSuccess) return internal_cuda_fail(e, "kernel launch");
    }
    const void* in = a;
    for (size_t i = 0; i < stages.size(); ++i) {
        const bool last = i + 1 == stages.size();
        void* out = last ? c : base + ((i & 1) ? off_d1 : off_d0);
        const Stage& sg = stages[i];
        const void* w = sg.group < 0 ? sg.w : base + off_w + ka.off[sg.group] * et;
        // the first stage follows the weights (if they go first), every later stage the
        // engine's previous kernel
        const bool dependent = i > 0 || ka.ngroups > 0;
        cudaError_t e = launch_plan(plans[i], in, w, out, base + off_part, st, &launches, dependent && !(i == 0 && weights_after));
        if (e != cudaSuccess) return internal_cuda_fail(e, "kernel launch");
        if (i == 0 && weights_after) {
            e = launch_weights(true);
            if (e != cudaSuccess) return internal_cuda_fail(e, "kernel launch");
        }
        in = out;
    }
    internal_count_launches(launches);
    return internal_ok();
}
