// C entry points over the reference library compiled from its own headers
// (TEST INFRASTRUCTURE ONLY: built into oracle/_ref/, never shipped).
//
// The reference is header-only C++17 (include/tlib/ttv.h and detail/*).  This
// file only instantiates its public call for every (execution, slicing,
// fusion) triple its own test-suite exercises (test/src/gtest_tlib_ttv.cpp)
// and its metadata helpers, and turns thrown std::runtime_error into a return
// code plus message, so Python tests can pin the oracle restatement against
// the real thing.  Build: oracle/Makefile, target _ref/libttvref.so, with
// -I pointing at the reference's include directory.
#include <tlib/ttv.h>

#include <cstring>
#include <stdexcept>
#include <vector>

using namespace tlib::ttv;

namespace {

void put_msg(char* msg, std::size_t len, const char* text)
{
    if (msg && len) {
        std::strncpy(msg, text, len - 1);
        msg[len - 1] = 0;
    }
}

template <class T, class E, class S, class F>
int call(E e, S s, F f, std::size_t q, std::size_t p, const T* a, const std::size_t* na,
         const std::size_t* wa, const std::size_t* pia, const T* b, const std::size_t* nb, T* c,
         const std::size_t* nc, const std::size_t* wc, const std::size_t* pic, char* msg,
         std::size_t len)
{
    try {
        ttv(e, s, f, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic);
    } catch (std::exception const& ex) {
        put_msg(msg, len, ex.what());
        return 1;
    }
    return 0;
}

template <class T>
int dispatch(int policy, std::size_t q, std::size_t p, const T* a, const std::size_t* na,
             const std::size_t* wa, const std::size_t* pia, const T* b, const std::size_t* nb,
             T* c, const std::size_t* nc, const std::size_t* wc, const std::size_t* pic,
             char* msg, std::size_t len)
{
    namespace ep = execution_policy;
    namespace sp = slicing_policy;
    namespace fp = fusion_policy;
#define REF_CALL(E, S, F) call<T>(E, S, F, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, msg, len)
    switch (policy) {
    case 0: return REF_CALL(ep::seq, sp::subtensor, fp::none);
    case 1: return REF_CALL(ep::par_loop, sp::subtensor, fp::all);
    case 2: return REF_CALL(ep::par_loop, sp::slice, fp::all);
    case 3: return REF_CALL(ep::seq, sp::slice, fp::none);
    case 4: return REF_CALL(ep::seq_blas, sp::subtensor, fp::none);
    case 5: return REF_CALL(ep::par, sp::subtensor, fp::none);
    case 6: return REF_CALL(ep::par_loop, sp::subtensor, fp::none);
    case 7: return REF_CALL(ep::par_task, sp::subtensor, fp::none);
    case 8: return REF_CALL(ep::par_taskloop, sp::subtensor, fp::none);
    case 9: return REF_CALL(ep::par_blas, sp::subtensor, fp::all);
    case 10: return REF_CALL(ep::seq_blas, sp::slice, fp::none);
    case 11: return REF_CALL(ep::par_task, sp::slice, fp::none);
    case 12: return REF_CALL(ep::par_taskloop, sp::slice, fp::none);
    case 13: return REF_CALL(ep::par, sp::slice, fp::none);
    case 14: return REF_CALL(ep::par_loop, sp::slice, fp::none);
    case 15: return REF_CALL(ep::par_loop, sp::slice, fp::outer);
    case 16: return REF_CALL(ep::par_blas, sp::slice, fp::all);
    default: put_msg(msg, len, "unknown policy"); return 2;
    }
#undef REF_CALL
}

} // namespace

extern "C" {

int ref_num_policies() { return 17; }

int ref_ttv_f32(int policy, std::size_t q, std::size_t p, const float* a, const std::size_t* na,
                const std::size_t* wa, const std::size_t* pia, const float* b,
                const std::size_t* nb, float* c, const std::size_t* nc, const std::size_t* wc,
                const std::size_t* pic, char* msg, std::size_t len)
{
    return dispatch<float>(policy, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, msg, len);
}

int ref_ttv_f64(int policy, std::size_t q, std::size_t p, const double* a, const std::size_t* na,
                const std::size_t* wa, const std::size_t* pia, const double* b,
                const std::size_t* nb, double* c, const std::size_t* nc, const std::size_t* wc,
                const std::size_t* pic, char* msg, std::size_t len)
{
    return dispatch<double>(policy, q, p, a, na, wa, pia, b, nb, c, nc, wc, pic, msg, len);
}

int ref_output_shape(const std::size_t* na, std::size_t p, std::size_t q, std::size_t* nc)
{
    try {
        std::vector<std::size_t> v(na, na + p);
        auto out = detail::generate_output_shape(v, q);
        std::copy(out.begin(), out.end(), nc);
    } catch (std::exception const&) {
        return 1;
    }
    return 0;
}

int ref_output_layout(const std::size_t* pia, std::size_t p, std::size_t q, std::size_t* pic)
{
    try {
        std::vector<std::size_t> v(pia, pia + p);
        auto out = detail::generate_output_layout(v, q);
        std::copy(out.begin(), out.end(), pic);
    } catch (std::exception const&) {
        return 1;
    }
    return 0;
}

int ref_strides(const std::size_t* n, const std::size_t* pi, std::size_t p, std::size_t* w)
{
    try {
        std::vector<std::size_t> vn(n, n + p), vp(pi, pi + p);
        auto out = detail::generate_strides(vn, vp);
        std::copy(out.begin(), out.end(), w);
    } catch (std::exception const&) {
        return 1;
    }
    return 0;
}

int ref_k_order_layout(std::size_t p, std::size_t k, std::size_t* pi)
{
    auto out = detail::generate_k_order_layout(p, k);
    std::copy(out.begin(), out.end(), pi);
    return 0;
}

int ref_is_valid_shape(const std::size_t* n, std::size_t len)
{
    return detail::is_valid_shape(n, n + len) ? 1 : 0;
}

int ref_is_valid_layout(const std::size_t* pi, std::size_t len)
{
    return detail::is_valid_layout(pi, pi + len) ? 1 : 0;
}

int ref_is_valid_strides(const std::size_t* pi, std::size_t len, const std::size_t* w)
{
    try {
        return detail::is_valid_strides(pi, pi + len, w) ? 1 : 0;
    } catch (std::exception const&) {
        return -1;
    }
}

std::size_t ref_inverse_mode(const std::size_t* pi, std::size_t p, std::size_t mode)
{
    return detail::inverse_mode(pi, pi + p, mode);
}

} // extern "C"
