// Device-side building blocks of the TTV kernels (sm_103a).
//
//  * vector loads of A in 16/8/4-byte units, streamed with evict-first hints
//  * fp32 compensated (Kahan) and plain accumulators, pairwise-compensated
//    combination of partial sums
//  * 1-D TMA bulk copy global -> shared (cp.async.bulk) completed on an
//    mbarrier, with a bounded wait that records a device error instead of
//    spinning forever
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tlibg {

// Device error word bits (each translation unit keeps its own word and
// passes its address): bit 0 = a bounded mbarrier wait expired.
constexpr unsigned ERR_WAIT_TIMEOUT = 1u;
// Upper bound of try_wait polls before a wait gives up (each poll may block
// for a hardware-defined slice; the bound is far above any legitimate copy).
constexpr uint32_t WAIT_POLL_LIMIT = 1u << 22;

// --------------------------------------------------------------------------
// programmatic dependent launch
// --------------------------------------------------------------------------
// First statement of every engine kernel.  `griddepcontrol.wait` returns at
// once unless the kernel was launched as a programmatic dependent of the
// previous kernel in its stream; then it blocks until that kernel has
// completed and its writes are visible, so nothing below it can read an
// input that is still being written or overwrite one still being read.
// `griddepcontrol.launch_dependents` lets a kernel launched as this one's
// programmatic dependent be scheduled once every CTA of this grid has issued
// it (so every CTA of this grid is already resident: a dependent that waits
// can never hold resources this grid still needs).  The host launches a
// kernel as a dependent only when its predecessor is the engine's own kernel
// of the same call (a combine after its main kernel, a chain stage after the
// one before); the dependent's launch then overlaps its predecessor's tail.
__device__ __forceinline__ void pdl_prologue()
{
    asm volatile("griddepcontrol.wait;\n\tgriddepcontrol.launch_dependents;" ::: "memory");
}

// --------------------------------------------------------------------------
// element conversion: A may be float, double or raw bfloat16 bits
// --------------------------------------------------------------------------
template <typename TA, typename T> struct Cvt;
template <> struct Cvt<float, float> {
    __device__ static float f(float x) { return x; }
};
template <> struct Cvt<double, double> {
    __device__ static double f(double x) { return x; }
};
template <> struct Cvt<uint16_t, float> {
    __device__ static float f(uint16_t x) { return __uint_as_float(((uint32_t)x) << 16); }
};

// Raw storage unit of V consecutive elements of TA (16, 8, 4 or 2 bytes).
template <int BYTES> struct RawVec;
template <> struct RawVec<16> { typedef uint4 type; };
template <> struct RawVec<8> { typedef uint2 type; };
template <> struct RawVec<4> { typedef uint32_t type; };
template <> struct RawVec<2> { typedef uint16_t type; };

// Streaming (read-once) load of V elements of A, converted to T.
template <typename TA, typename T, int V>
__device__ __forceinline__ void load_a(const TA* p, T (&out)[V])
{
    constexpr int B = (int)sizeof(TA) * V;
    typedef typename RawVec<B>::type R;
    R r = __ldcs(reinterpret_cast<const R*>(p));
    const TA* e = reinterpret_cast<const TA*>(&r);
#pragma unroll
    for (int v = 0; v < V; ++v) out[v] = Cvt<TA, T>::f(e[v]);
}
// The same through L1 (read-only path, default caching): for access
// patterns where one thread reads consecutive vectors of a line that other
// lanes do not share (one lane per row), so the second half of each 32-byte
// sector is still in L1 when the thread's next load asks for it.
template <typename TA, typename T, int V>
__device__ __forceinline__ void load_a_l1(const TA* p, T (&out)[V])
{
    constexpr int B = (int)sizeof(TA) * V;
    typedef typename RawVec<B>::type R;
    R r = __ldg(reinterpret_cast<const R*>(p));
    const TA* e = reinterpret_cast<const TA*>(&r);
#pragma unroll
    for (int v = 0; v < V; ++v) out[v] = Cvt<TA, T>::f(e[v]);
}

template <> __device__ __forceinline__ void load_a<uint16_t, float, 1>(const uint16_t* p, float (&out)[1])
{
    unsigned short r;
    asm volatile("ld.global.cs.u16 %0, [%1];" : "=h"(r) : "l"(p));
    out[0] = __uint_as_float(((uint32_t)r) << 16);
}

// --------------------------------------------------------------------------
// accumulators.  Value represented = s - c (c carries the negated error).
// --------------------------------------------------------------------------
template <typename T, bool KAHAN> struct Acc {
    T s, c;
    __device__ __forceinline__ void init() { s = T(0); c = T(0); }
    __device__ __forceinline__ void fma_add(T a, T b)
    {
        if (KAHAN) {
            T y = fma(a, b, -c);     // product minus the running compensation
            T t = s + y;
            c = (t - s) - y;         // what was lost adding y to s
            s = t;
        } else {
            s = fma(a, b, s);
        }
    }
    // Combine with another accumulator (order-fixed, compensated).
    __device__ __forceinline__ void merge(T os, T oc)
    {
        if (KAHAN) {
            T t = s + os;                      // two-sum of the two leading parts
            T bp = t - s;
            T e = (s - (t - bp)) + (os - bp);  // exact rounding error of s + os
            c = (c + oc) - e;
            s = t;
        } else {
            s = s + os;
        }
    }
    __device__ __forceinline__ T value() const { return KAHAN ? (s - c) : s; }
    __device__ __forceinline__ void renorm() {}
    __device__ __forceinline__ void fold() {}
};

// --------------------------------------------------------------------------
// fp64 products accumulated on the FP32 / INT32 pipes.
//
// GB300 executes about two DFMA per SM per clock (1.25 TFLOP/s), below the
// one-per-element rate an HBM-bound fp64 TTV needs.  Each double x with
// exponent in [2^-60, 2^61) is split into x ~ hi + lo with integer ops and
// one FP32 add: hi = x cut to its top 24 significand bits (one funnel shift
// moves the significand into float position, one add rebiases the exponent
// modulo 256, one bit-select restores the sign); lo = the next 23 bits, built
// as the float 1.m * 2^(e-1046) minus 2^(e-1046) (exact).  The 6 lowest
// significand bits are dropped: |x - hi - lo| < 2^-46 |x|.  No int -> float
// conversion is used: on this part those issue at the FP64 pipe's rate.  The
// product a*b = hi_a*hi_b + (hi_a*lo_b + lo_a*hi_b) keeps hi_a*hi_b exact
// through Dekker's TwoProduct (one FMA gives its rounding error); lo_a*lo_b
// (below 2^-48 of the product) is dropped.  The running sum is a double-float
// (hi, lo): Knuth's TwoSum adds each product to hi exactly and the error goes
// to lo; renorm() (every few products, and before fold()) moves lo's excess
// back into hi so lo's own rounding stays near 2^-48 of the sum.  Elements
// outside the exponent window (zeros, subnormals, non-finite values) take a
// native DFMA into a separate double accumulator.  fold() turns the state
// into one double, in `s`, before any cross-lane or cross-warp reduction.
// --------------------------------------------------------------------------
struct DSplit {
    float hi, lo;
    bool ok;
};

__device__ __forceinline__ DSplit split_double(double x)
{
    const uint32_t hi32 = (uint32_t)__double2hiint(x), lo32 = (uint32_t)__double2loint(x);
    DSplit r;
    // biased exponent e in [963, 1083]: 2^-60 <= |x| < 2^61
    r.ok = ((hi32 & 0x7ff00000u) - (963u << 20)) < (121u << 20);
    // top 32 bits of (hi32:lo32) << 3 hold e mod 256 and 23 significand bits;
    // float exponent e - 896 == (e mod 256) + 128 (mod 256) inside the window
    const uint32_t top = __funnelshift_l(lo32, hi32, 3) + (128u << 23);
    const uint32_t hb = (top & 0x7fffffffu) | (hi32 & 0x80000000u);
    r.hi = __uint_as_float(hb);
    // +-2^(e-1046) (hi's sign and exponent field minus 23; the field is at
    // least 67, so nothing borrows from the sign); the same with significand
    // bits 28..6 of x is +-(1 + f/2^23) 2^(e-1046), and the difference of the
    // two is exact (Sterbenz): +-f 2^(e-1069), the next 23 bits of x
    const uint32_t sgnexp = (hb & 0xff800000u) - (23u << 23);
    r.lo = __uint_as_float(sgnexp | ((lo32 >> 6) & 0x7fffffu)) - __uint_as_float(sgnexp);
    return r;
}

// Out-of-window products: a real call, so the compiler cannot turn the rare
// branch into a predicated DFMA that would take an FP64 issue slot for every
// in-window product as well.
static __device__ __noinline__ double dfma_out_of_window(double a, double b, double d) { return fma(a, b, d); }
static __device__ __noinline__ double f2d_convert(float x) { return (double)x; }

// float -> double without the conversion instruction (it issues at the FP64
// pipe's rate here): for a normal float the double's high word is the
// float's magnitude bits shifted right by 3 plus the exponent rebias
// (1023 - 127) << 20, with the sign kept; the low word holds the last 3
// significand bits.  Zeros are built directly; subnormal and non-finite
// floats take the conversion through a real call (never predicated in).
__device__ __forceinline__ double f2d(float x)
{
    const uint32_t u = __float_as_uint(x);
    const uint32_t m = u & 0x7fffffffu;
    if (m - 0x00800000u < 0x7f000000u)
        return __hiloint2double((int)(((m >> 3) + (896u << 20)) | (u & 0x80000000u)), (int)(u << 29));
    if (m == 0) return __hiloint2double((int)(u & 0x80000000u), 0);
    return f2d_convert(x);
}

struct AccDF {
    double s, c;    // folded value (after fold()); c stays 0
    float hi, lo;   // double-float running sum
    double d;       // native DFMA accumulator for out-of-window elements
    __device__ __forceinline__ void init()
    {
        s = 0.0;
        c = 0.0;
        hi = 0.f;
        lo = 0.f;
        d = 0.0;
    }
    // One product into the running sum, without renormalisation: callers
    // renorm() at least every 8 products.
    __device__ __forceinline__ void add_split(const DSplit& a, const DSplit& b, double ad, double bd)
    {
        if (a.ok && b.ok) {
            const float p = a.hi * b.hi;
            const float t = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
            const float sum = hi + p;                                           // TwoSum(hi, p)
            const float v = sum - hi;
            lo += ((hi - (sum - v)) + (p - v)) + t;
            hi = sum;
        } else {
            d = dfma_out_of_window(ad, bd, d);
        }
    }
    __device__ __forceinline__ void renorm()
    {
        const float sum = hi + lo;
        lo -= sum - hi;
        hi = sum;
    }
    __device__ __forceinline__ void fma_add(double a, double b)
    {
        add_split(split_double(a), split_double(b), a, b);
        renorm();
    }
    __device__ __forceinline__ void fold()
    {
        renorm();
        s = (f2d(hi) + f2d(lo)) + d;
        c = 0.0;
    }
    __device__ __forceinline__ void merge(double os, double) { s = s + os; }
    __device__ __forceinline__ double value() const { return s; }
    // Take over another (unfolded) accumulator of the same output: the
    // double-floats merge on the FP32 pipe (TwoSum), only the DFMA parts
    // need one DADD.
    __device__ __forceinline__ void absorb(const AccDF& o)
    {
        const float sum = hi + o.hi;
        const float v = sum - hi;
        lo += ((hi - (sum - v)) + (o.hi - v)) + o.lo;
        hi = sum;
        d += o.d;
    }
};

// Reduce the V accumulators of one lane (parts of the same dot product) into
// acc[0], folded.
template <int V, typename T, bool KAHAN> __device__ __forceinline__ void fold_vec(Acc<T, KAHAN> (&acc)[V])
{
#pragma unroll
    for (int v = 1; v < V; ++v) acc[0].merge(acc[v].s, acc[v].c);
}
template <int V> __device__ __forceinline__ void fold_vec(AccDF (&acc)[V])
{
#pragma unroll
    for (int v = 1; v < V; ++v) acc[0].absorb(acc[v]);
    acc[0].fold();
}

// Accumulator of a kernel instantiation: fp32 plain / Kahan, fp64 native
// DFMA (KAHAN == false) or double-float emulation (KAHAN == true).
template <typename T, bool KAHAN> struct AccSel {
    typedef Acc<T, KAHAN> type;
};
template <> struct AccSel<double, true> {
    typedef AccDF type;
};

// --------------------------------------------------------------------------
// mbarrier + 1-D TMA bulk copy
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// dst and src 16-byte aligned, bytes a positive multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait; false (and the device error word set) if the phase never
// completed within `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, unsigned int* err,
                                                  uint32_t limit = WAIT_POLL_LIMIT)
{
    for (uint32_t it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(err, ERR_WAIT_TIMEOUT);
    return false;
}

// Stage b[ib, ie) into shared memory so that element e lands at
//   smem_b[off + (e - ib)],   off = ((uintptr)(b + ib) % 16) / sizeof(T),
// i.e. shared and global addresses agree modulo 16.  The 16-byte-aligned body
// moves with one TMA bulk copy issued by thread 0; the ragged head and tail
// (at most 15 bytes each) are plain loads.  Must be called by the whole CTA;
// returns false on an expired wait (all threads then leave the kernel).
template <typename T>
__device__ __forceinline__ bool stage_b(T* smem_b, const T* b, uint64_t ib, uint64_t ie,
                                        uint64_t* bar, uint32_t& phase, int* abort_flag,
                                        unsigned int* err)
{
    const uintptr_t g0 = reinterpret_cast<uintptr_t>(b + ib);
    const uintptr_t g1 = reinterpret_cast<uintptr_t>(b + ie);
    const uintptr_t body0 = (g0 + 15) & ~uintptr_t(15);
    uintptr_t body1 = g1 & ~uintptr_t(15);
    if (body1 < body0) body1 = body0;
    const uint32_t off = (uint32_t)((g0 & 15) / sizeof(T));
    const uint32_t body_bytes = (uint32_t)(body1 - body0);
    const uint64_t head_n = (body0 - g0) / sizeof(T) < (ie - ib) ? (body0 - g0) / sizeof(T) : (ie - ib);
    const uint64_t body_first = ib + head_n;                     // first element of the body
    const uint64_t tail_first = body_first + body_bytes / sizeof(T);

    if (threadIdx.x == 0) {
        fence_proxy_async_smem();   // order earlier generic reads of smem_b before the async write
        mbar_arrive_expect_tx(bar, body_bytes);
        if (body_bytes) bulk_g2s(smem_b + off + head_n, b + body_first, body_bytes, bar);
    }
    for (uint64_t e = ib + threadIdx.x; e < body_first; e += blockDim.x) smem_b[off + (e - ib)] = __ldg(b + e);
    for (uint64_t e = tail_first + threadIdx.x; e < ie; e += blockDim.x) smem_b[off + (e - ib)] = __ldg(b + e);
    if (threadIdx.x == 0) {
        if (!mbar_wait_bounded(bar, phase, err)) {
            *abort_flag = 1;
            // give an in-flight copy a second bounded chance to land before leaving.
            // No further copy is issued after an expiry: the caller returns.  If this
            // wait expires too, the CTA leaves with at most this one copy outstanding
            // (its destination is this CTA's shared memory); the device error word is
            // set, the host reports TLIBG_ERR_TIMEOUT and the results (and any later
            // work sharing that SM's shared memory) must be treated as invalid.
            mbar_wait_bounded(bar, phase, err);
        }
    }
    phase ^= 1u;
    __syncthreads();
    return *abort_flag == 0;
}

}  // namespace tlibg
