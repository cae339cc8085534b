/*
 * tlib/ttv_gpu.h -- GB300 execution policies for tlib's tensor-times-vector.
 *
 * Drop-in for the reference's low-level call
 *     tlib::ttv::ttv(ep, sp, fp, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic)
 * (reference include/tlib/ttv.h:54-92): pass one of the policies below as
 * `ep` and device pointers as a, b, c.  The reference's validation runs
 * first (same checks, same exception text); its dispatch to detail::ttv
 * (tensor_times_vector.h:416-421) then resolves to the overloads declared
 * here, which call the engine through its C ABI (tlibg.h).
 *
 *   execution_policy::gpu          synchronous: C is complete on return,
 *                                  like every CPU policy of the reference
 *   execution_policy::gpu_on(s)    enqueue on CUDA stream s, return at once
 *
 * Any slicing_policy / fusion_policy tag is accepted; the engine always fuses
 * every free mode into one grid (the reference's fusion_policy::all).  When
 * a, b and c are all host pointers (for instance the data of the reference's
 * own tensor<T>, so that its high-level ttv(q, A, b, gpu, ...) works as is),
 * the call takes the engine's host path and is synchronous.
 *
 * tlib/ttv_gpu_tensor.h adds a device-resident tensor with the reference's
 * tensor / tensor_view / A(q) * b interface.
 *
 * Include this header INSTEAD OF (or before) <tlib/ttv.h>: the reference
 * dispatches through a qualified call, so the overloads must be declared
 * before its templates are defined.  Where the reference headers are not on
 * the include path, the header provides the same low-level entry point and
 * policy tag names by itself (standalone mode) so code written against
 * tlib's low-level interface compiles unchanged.
 */
#pragma once

#include <cstddef>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../tlibg.h"

#if __has_include(<tlib/detail/tags.h>) && !defined(TLIBG_STANDALONE)
#include <tlib/detail/tags.h>
#define TLIBG_WITH_REFERENCE 1
#else
// Standalone mode: the policy tag names of tlib (reference detail/tags.h),
// so call sites written for the reference compile without it.
namespace tlib::ttv::execution_policy {
struct sequential_t {};
struct parallel_loop_t {};
inline constexpr sequential_t seq;
inline constexpr parallel_loop_t par_loop;
}  // namespace tlib::ttv::execution_policy
namespace tlib::ttv::slicing_policy {
struct slice_t {};
struct subtensor_t {};
inline constexpr slice_t slice;
inline constexpr subtensor_t subtensor;
}  // namespace tlib::ttv::slicing_policy
namespace tlib::ttv::fusion_policy {
struct none_t {};
struct outer_t {};
struct all_t {};
inline constexpr none_t none;
inline constexpr outer_t outer;
inline constexpr all_t all;
}  // namespace tlib::ttv::fusion_policy
#define TLIBG_WITH_REFERENCE 0
#endif

namespace tlib::ttv::execution_policy {
struct gpu_t {};
struct gpu_stream_t {
    void* stream;
};
inline constexpr gpu_t gpu;
inline gpu_stream_t gpu_on(void* stream) { return gpu_stream_t{stream}; }
}  // namespace tlib::ttv::execution_policy

namespace tlib::ttv::gpu_detail {

inline void throw_status(int status)
{
    if (status == TLIBG_OK) return;
    char buf[1024];
    tlibg_last_error(buf, sizeof(buf));
    throw std::runtime_error(std::string(buf));
}

template <class value_t> constexpr int dtype_of()
{
    static_assert(std::is_same_v<value_t, float> || std::is_same_v<value_t, double>,
                  "the gpu policies support float and double");
    return std::is_same_v<value_t, float> ? TLIBG_F32 : TLIBG_F64;
}

// size arrays as std::size_t, converting other index types once
template <class size_type> struct Sizes {
    std::vector<std::size_t> buf;
    const std::size_t* ptr = nullptr;
    Sizes(const size_type* v, std::size_t n)
    {
        if constexpr (std::is_same_v<size_type, std::size_t>) {
            ptr = v;
        } else if (v) {
            buf.assign(v, v + n);
            ptr = buf.data();
        }
    }
};

// Device pointers run on the device (asynchronously for gpu_on); when a, b
// and c all live in host memory -- the reference's own tensor<T> keeps its
// data in a std::vector -- the call goes through the engine's host path
// (copies in, computes on the GPU, copies C back; synchronous either way).
template <class value_t, class size_type>
inline void run(void* stream, bool sync, std::size_t q, std::size_t p, const value_t* a,
                const size_type* na, const size_type* wa, const size_type* pia, const value_t* b,
                const size_type* nb, value_t* c, const size_type* nc, const size_type* wc,
                const size_type* pic)
{
    const std::size_t pc = p ? p - 1 : 0;
    Sizes<size_type> sna(na, p), swa(wa, p), spia(pia, p), snb(nb, 1), snc(nc, pc), swc(wc, pc),
        spic(pic, pc);
    tlibg_options opt{TLIBG_ACC_COMPENSATED, -1, 0, 0, 0, sync ? 1 : 0};
    if (a && b && c && tlibg_pointer_location(a) == 0 && tlibg_pointer_location(b) == 0 &&
        tlibg_pointer_location(c) == 0) {
        throw_status(tlibg_ttv_host(dtype_of<value_t>(), q, p, a, sna.ptr, swa.ptr, spia.ptr, b,
                                    snb.ptr, c, snc.ptr, swc.ptr, spic.ptr, &opt));
        return;
    }
    throw_status(tlibg_ttv_ex(dtype_of<value_t>(), q, p, a, sna.ptr, swa.ptr, spia.ptr, b, snb.ptr,
                              c, snc.ptr, swc.ptr, spic.ptr, &opt, stream));
}

}  // namespace tlib::ttv::gpu_detail

namespace tlib::ttv::detail {

// Overloads picked by the reference's dispatch (tensor_times_vector.h:416-421)
template <class value_t, class size_type, class slicing_t, class fusion_t>
inline void ttv(execution_policy::gpu_t, slicing_t, fusion_t, unsigned const m, unsigned const p,
                value_t const* const a, size_type const* const na, size_type const* const wa,
                size_type const* const pia, value_t const* const b, size_type const* const nb,
                value_t* const c, size_type const* const nc, size_type const* const wc,
                size_type const* const pic)
{
    gpu_detail::run(nullptr, true, m, p, a, na, wa, pia, b, nb, c, nc, wc, pic);
}

template <class value_t, class size_type, class slicing_t, class fusion_t>
inline void ttv(execution_policy::gpu_stream_t ep, slicing_t, fusion_t, unsigned const m,
                unsigned const p, value_t const* const a, size_type const* const na,
                size_type const* const wa, size_type const* const pia, value_t const* const b,
                size_type const* const nb, value_t* const c, size_type const* const nc,
                size_type const* const wc, size_type const* const pic)
{
    gpu_detail::run(ep.stream, false, m, p, a, na, wa, pia, b, nb, c, nc, wc, pic);
}

}  // namespace tlib::ttv::detail

#if TLIBG_WITH_REFERENCE
#include <tlib/ttv.h>
#else
namespace tlib::ttv {
// The low-level entry point of the reference (ttv.h:54-92) for the gpu
// policies.  The engine performs the reference's argument checks itself, in
// the same order and with the same messages, and throws std::runtime_error.
template <class value_t, class size_type, class execution_t, class slicing_t, class fusion_t>
inline void ttv(execution_t ep, slicing_t sp, fusion_t fp, size_type const q, size_type const p,
                value_t const* const a, size_type const* const na, size_type const* const wa,
                size_type const* const pia, value_t const* const b, size_type const* const nb,
                value_t* const c, size_type const* const nc, size_type const* const wc,
                size_type const* const pic)
{
    static_assert(std::is_same_v<execution_t, execution_policy::gpu_t> ||
                      std::is_same_v<execution_t, execution_policy::gpu_stream_t>,
                  "standalone tlib/ttv_gpu.h provides the gpu execution policies only");
    if constexpr (std::is_same_v<execution_t, execution_policy::gpu_t>)
        gpu_detail::run(nullptr, true, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic);
    else
        gpu_detail::run(ep.stream, false, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic);
    (void)sp;
    (void)fp;
}
}  // namespace tlib::ttv
#endif

namespace tlib::ttv::gpu {

// A stored as bfloat16 (raw 16-bit patterns), b and C float; no reference
// counterpart for the storage type, same argument meaning as ttv.h:54-60.
template <class size_type>
inline void ttv_bf16a(size_type q, size_type p, const uint16_t* a, const size_type* na,
                      const size_type* wa, const size_type* pia, const float* b,
                      const size_type* nb, float* c, const size_type* nc, const size_type* wc,
                      const size_type* pic, void* stream = nullptr, bool sync = true)
{
    const std::size_t pc = p ? p - 1 : 0;
    gpu_detail::Sizes<size_type> sna(na, p), swa(wa, p), spia(pia, p), snb(nb, 1), snc(nc, pc),
        swc(wc, pc), spic(pic, pc);
    tlibg_options opt{TLIBG_ACC_COMPENSATED, -1, 0, 0, 0, sync ? 1 : 0};
    gpu_detail::throw_status(tlibg_ttv_ex(TLIBG_BF16A, q, p, a, sna.ptr, swa.ptr, spia.ptr, b,
                                          snb.ptr, c, snc.ptr, swc.ptr, spic.ptr, &opt, stream));
}

}  // namespace tlib::ttv::gpu
