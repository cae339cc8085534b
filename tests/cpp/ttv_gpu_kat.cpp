// Known-answer test of the gpu execution policy through tlib's low-level call
// (restates the check of the reference's test/src/gtest_tlib_ttv.cpp:28-140:
// A holds 1, 2, 3, ... along mode q, b = 1, so every output j is a sum of n_q
// consecutive integers, (n_q^2 (2i - 1) + n_q) / 2 with i = j + 1).
//
//   ttv_gpu_kat validate   argument errors only (no device needed): the
//                          exception text equals the reference's
//   ttv_gpu_kat kat        the KAT grid on the GPU (ranks 2-4, extents
//                          {2, 4, 8}, every layout and q), float and double,
//                          each call with one of the six (slicing, fusion)
//                          pairs of the reference's tests in turn
//   ttv_gpu_kat tensor     the device tensor interface (A(q) * b, ttv(q, A, b))
//                          on the KAT grid of rank 3, host-pointer calls of the
//                          gpu policy, and (with the reference headers) the
//                          reference's own tensor<T> through the gpu policy
//
// Built with the reference headers on the include path (the policy hooks into
// the reference's own dispatch) or without them (standalone mode).
#include <tlib/ttv_gpu.h>
#include <tlib/ttv_gpu_tensor.h>

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

using namespace tlib::ttv;
using sizes = std::vector<std::size_t>;

static int failures = 0;

static sizes out_shape(const sizes& na, std::size_t q)
{
    sizes nc(na.size() - 1);
    tlibg_output_shape(na.data(), na.size(), q, nc.data());
    return nc;
}
static sizes out_layout(const sizes& pia, std::size_t q)
{
    sizes pic(pia.size() - 1);
    tlibg_output_layout(pia.data(), pia.size(), q, pic.data());
    return pic;
}
static sizes dense(const sizes& n, const sizes& pi)
{
    sizes w(n.size());
    tlibg_strides(n.data(), pi.data(), n.size(), w.data());
    return w;
}

static void expect_throw(const char* what, const std::string& expected, std::size_t q, std::size_t p,
                         const float* a, sizes na, sizes wa, sizes pia, const float* b, sizes nb,
                         float* c, sizes nc, sizes wc, sizes pic)
{
    try {
        ttv(execution_policy::gpu, slicing_policy::subtensor, fusion_policy::all, q, p, a,
            na.data(), wa.data(), pia.data(), b, nb.data(), c, nc.data(), wc.data(), pic.data());
        std::printf("FAIL %s: no exception\n", what);
        ++failures;
    } catch (std::runtime_error const& e) {
        if (expected.empty() ? std::strlen(e.what()) == 0 : std::string(e.what()).find(expected) == std::string::npos) {
            std::printf("FAIL %s: got '%s'\n", what, e.what());
            ++failures;
        }
    }
}

static int validate()
{
    float dummy[64] = {};
    const float* a = dummy;
    const float* b = dummy;
    float* c = dummy;
    sizes na{2, 3, 4}, pia{1, 2, 3}, wa{1, 2, 6}, nb{3}, nc{2, 4}, pic{1, 2}, wc{1, 2};
    const std::string E = "Error in tlib::tensor_times_vector: ";
    expect_throw("q", E + "contraction mode should be greater zero or less than or equal to p.", 4, 3, a, na, wa, pia, b, nb, c, nc, wc, pic);
    expect_throw("nb", E + "contraction dimension of A and B are not equal.", 2, 3, a, na, wa, pia, b, sizes{5}, c, nc, wc, pic);
    expect_throw("A null", E + "pointer to input tensor A should not be zero.", 2, 3, nullptr, na, wa, pia, b, nb, c, nc, wc, pic);
    expect_throw("pia", E + "layout vector of A is not valid.", 2, 3, a, na, wa, sizes{1, 1, 3}, b, nb, c, nc, wc, pic);
    expect_throw("wa", E + "stride vector of A is not valid.", 2, 3, a, na, sizes{1, 8, 2}, pia, b, nb, c, nc, wc, pic);
    expect_throw("pic", "Error in tlib::detail::compute_inverse_pia_m: beginning of layout tuples of both tensors are not correct.",
                 2, 3, a, na, wa, pia, b, nb, c, nc, sizes{4, 1}, sizes{2, 1});
    // device tensor: the reference's constructor and call-operator checks
    const std::string T = "Error in tlib::tensor: ";
    auto expect_tensor_throw = [&](const char* what, const std::string& expected, auto&& make) {
        try {
            make();
            std::printf("FAIL %s: no exception\n", what);
            ++failures;
        } catch (std::runtime_error const& e) {
            if (std::string(e.what()).find(expected) == std::string::npos) {
                std::printf("FAIL %s: got '%s'\n", what, e.what());
                ++failures;
            }
        }
    };
    expect_tensor_throw("tensor lengths", T + "shape vector and layout vector must have the same length.",
                        [] { tlib::ttv::gpu::tensor<float> x(sizes{2, 3}, sizes{1}); });
    expect_tensor_throw("tensor shape", T + "shape vector of tensor is not valid.",
                        [] { tlib::ttv::gpu::tensor<float> x(sizes{2, 0}, sizes{1, 2}); });
    expect_tensor_throw("tensor layout", T + "layout vector of tensor is not valid.",
                        [] { tlib::ttv::gpu::tensor<float> x(sizes{2, 3}, sizes{2, 2}); });
    // a valid call reaches the engine (host memory is not device memory: the
    // engine refuses without touching it when no device is present)
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        expect_throw("valid call without a device", "tlibg: no usable CUDA device", 2, 3, a, na, wa, pia, b, nb, c, nc, wc, pic);
    std::printf("%s validate (%s)\n", failures ? "FAILED" : "PASSED",
                TLIBG_WITH_REFERENCE ? "reference headers" : "standalone");
    return failures ? 1 : 0;
}

template <class T>
static void init_kat(std::size_t q, std::vector<T>& a, const sizes& na, const sizes& wa, const sizes& pia)
{
    // walk the layout outermost-first with mode q innermost, numbering 1, 2, ...
    const std::size_t p = na.size();
    std::size_t q1 = 0;
    while (pia[q1] != q) ++q1;
    sizes order;
    for (std::size_t r = p; r-- > 0;)
        if (r != q1) order.push_back(pia[r] - 1);
    order.push_back(q - 1);
    sizes idx(p, 0);
    std::size_t k = 0;
    const std::size_t total = std::accumulate(na.begin(), na.end(), std::size_t(1), std::multiplies<>());
    for (std::size_t t = 0; t < total; ++t) {
        std::size_t off = 0;
        for (std::size_t r = 0; r < p; ++r) off += idx[r] * wa[r];
        a[off] = T(++k);
        for (std::size_t d = order.size(); d-- > 0;) {
            const std::size_t m = order[d];
            if (++idx[m] < na[m]) break;
            idx[m] = 0;
        }
    }
}

// The low-level call through the gpu policy with slicing / fusion pair k of
// {slice, subtensor} x {none, outer, all}: the engine treats them as the
// scheduling hints they are on the CPU and computes the same C.
static std::size_t pair_index = 0;
static std::size_t pair_seen[6] = {};

template <class T>
static void call_with_pair(std::size_t k, std::size_t q, std::size_t p, const T* a, const sizes& na,
                           const sizes& wa, const sizes& pia, const T* b, const sizes& nb, T* c,
                           const sizes& nc, const sizes& wc, const sizes& pic)
{
    ++pair_seen[k];
    const auto ep = execution_policy::gpu;
    const auto* n = na.data();
    switch (k) {
    case 0: ttv(ep, slicing_policy::subtensor, fusion_policy::all, q, p, a, n, wa.data(), pia.data(), b, nb.data(), c, nc.data(), wc.data(), pic.data()); break;
    case 1: ttv(ep, slicing_policy::subtensor, fusion_policy::none, q, p, a, n, wa.data(), pia.data(), b, nb.data(), c, nc.data(), wc.data(), pic.data()); break;
    case 2: ttv(ep, slicing_policy::subtensor, fusion_policy::outer, q, p, a, n, wa.data(), pia.data(), b, nb.data(), c, nc.data(), wc.data(), pic.data()); break;
    case 3: ttv(ep, slicing_policy::slice, fusion_policy::all, q, p, a, n, wa.data(), pia.data(), b, nb.data(), c, nc.data(), wc.data(), pic.data()); break;
    case 4: ttv(ep, slicing_policy::slice, fusion_policy::none, q, p, a, n, wa.data(), pia.data(), b, nb.data(), c, nc.data(), wc.data(), pic.data()); break;
    default: ttv(ep, slicing_policy::slice, fusion_policy::outer, q, p, a, n, wa.data(), pia.data(), b, nb.data(), c, nc.data(), wc.data(), pic.data()); break;
    }
}

template <class T>
static int kat_rank(std::size_t rank)
{
    sizes ext{2, 4, 8};
    std::vector<sizes> shapes(1);
    for (std::size_t r = 0; r < rank; ++r) {
        std::vector<sizes> next;
        for (auto& s : shapes)
            for (auto e : ext) {
                auto t = s;
                t.push_back(e);
                next.push_back(t);
            }
        shapes = next;
    }
    sizes perm(rank);
    std::iota(perm.begin(), perm.end(), 1);
    std::vector<sizes> layouts;
    do layouts.push_back(perm);
    while (std::next_permutation(perm.begin(), perm.end()));

    int bad = 0;
    for (auto& na : shapes) {
        const std::size_t nn = std::accumulate(na.begin(), na.end(), std::size_t(1), std::multiplies<>());
        std::vector<T> a(nn);
        T *da, *db, *dc;
        cudaMalloc(&da, nn * sizeof(T));
        cudaMalloc(&db, 8 * sizeof(T));
        cudaMalloc(&dc, nn * sizeof(T));
        for (auto& pia : layouts) {
            const sizes wa = dense(na, pia);
            for (std::size_t q = 1; q <= rank; ++q) {
                init_kat(q, a, na, wa, pia);
                std::vector<T> b(na[q - 1], T(1));
                const sizes nc = out_shape(na, q), pic = out_layout(pia, q), wc = dense(nc, pic);
                const sizes nb{na[q - 1]};
                cudaMemcpy(da, a.data(), nn * sizeof(T), cudaMemcpyHostToDevice);
                cudaMemcpy(db, b.data(), b.size() * sizeof(T), cudaMemcpyHostToDevice);
                // every (slicing, fusion) pair the reference's own tests pass
                // (gtest_tlib_ttv.cpp:192-425), in turn over the grid's calls
                call_with_pair(pair_index++ % 6, q, rank, da, na, wa, pia, db, nb, dc, nc, wc, pic);
                const std::size_t ncn = nn / na[q - 1];
                std::vector<T> c(ncn);
                cudaMemcpy(c.data(), dc, ncn * sizeof(T), cudaMemcpyDeviceToHost);
                // C's elements in its own layout order are outputs 1, 2, 3, ...
                const std::size_t nq = na[q - 1];
                sizes idx(rank - 1, 0);
                for (std::size_t t = 0; t < ncn; ++t) {
                    std::size_t off = 0;
                    for (std::size_t r = 0; r + 1 < rank; ++r) off += idx[r] * wc[r];
                    const std::size_t i = t + 1;
                    const T want = T((nq * nq * (2 * i - 1) + nq) / 2);
                    if (c[off] != want) {
                        if (bad < 5) std::printf("KAT mismatch rank %zu q %zu: got %g want %g\n", rank, q, double(c[off]), double(want));
                        ++bad;
                    }
                    for (std::size_t d = 0; d + 1 < rank; ++d) {
                        const std::size_t m = pic[d] - 1;
                        if (++idx[m] < nc[m]) break;
                        idx[m] = 0;
                    }
                }
            }
        }
        cudaFree(da);
        cudaFree(db);
        cudaFree(dc);
    }
    return bad;
}

// The device tensor interface on the rank-3 KAT grid, the gpu policy on host
// pointers, and the reference's own tensor<T> through the gpu policy.
template <class T>
static int tensor_api()
{
    using gt = tlib::ttv::gpu::tensor<T>;
    int bad = 0;
    sizes perm{1, 2, 3};
    do {
        for (std::size_t q = 1; q <= 3; ++q) {
            const sizes na{4, 2, 8};
            const sizes wa = dense(na, perm);
            std::vector<T> a(64);
            init_kat(q, a, na, wa, perm);
            gt A(na, perm, a);
            gt b(sizes{na[q - 1]});
            b = T(1);
            for (int form = 0; form < 3; ++form) {
                gt C = form == 0 ? A(q) * b : tlib::ttv::gpu::ttv(q, A, b);
                std::vector<T> c = C.to_host();
                if (form == 2) {
                    // host pointers through the gpu policy: the engine's host path
                    std::vector<T> bh(na[q - 1], T(1));
                    const sizes nc = C.shape(), pic = C.layout(), wc = C.strides(), nb{na[q - 1]};
                    std::fill(c.begin(), c.end(), T(-1));
                    ttv(execution_policy::gpu, slicing_policy::subtensor, fusion_policy::all, q, std::size_t(3),
                        a.data(), na.data(), wa.data(), perm.data(), bh.data(), nb.data(), c.data(), nc.data(),
                        wc.data(), pic.data());
                }
                // C's elements in its own layout order are outputs 1, 2, 3, ...
                const sizes nc = C.shape(), pic = C.layout(), wc = C.strides();
                const std::size_t nq = na[q - 1];
                sizes idx(2, 0);
                for (std::size_t t = 0; t < c.size(); ++t) {
                    const std::size_t off = idx[0] * wc[0] + idx[1] * wc[1];
                    const std::size_t i = t + 1;
                    const T want = T((nq * nq * (2 * i - 1) + nq) / 2);
                    if (c[off] != want) {
                        if (bad < 5) std::printf("tensor mismatch form %d q %zu: got %g want %g\n", form, q, double(c[off]), double(want));
                        ++bad;
                    }
                    for (std::size_t d = 0; d < 2; ++d) {
                        const std::size_t m = pic[d] - 1;
                        if (++idx[m] < nc[m]) break;
                        idx[m] = 0;
                    }
                }
            }
        }
    } while (std::next_permutation(perm.begin(), perm.end()));
#if TLIBG_WITH_REFERENCE
    // the reference's own high-level call with its host tensor<T> and the gpu policy
    tlib::ttv::tensor<T> Ah({4, 2, 8}, {1, 2, 3}), bh({2});
    std::iota(Ah.begin(), Ah.end(), T(1));
    std::fill(bh.begin(), bh.end(), T(1));
    auto Ch = tlib::ttv::ttv(2, Ah, bh, execution_policy::gpu, slicing_policy::subtensor, fusion_policy::all);
    auto Cr = tlib::ttv::ttv(2, Ah, bh, execution_policy::seq, slicing_policy::subtensor, fusion_policy::none);
    if (!std::equal(Ch.begin(), Ch.end(), Cr.begin())) {
        std::printf("reference tensor<T> through the gpu policy differs from its seq policy\n");
        ++bad;
    }
    gt Ad(Ah);
    auto Cd = (Ad(2) * gt(bh)).host();
    if (!std::equal(Cd.begin(), Cd.end(), Cr.begin())) {
        std::printf("device tensor made from the reference's tensor<T> differs\n");
        ++bad;
    }
#endif
    return bad;
}

int main(int argc, char** argv)
{
    const std::string mode = argc > 1 ? argv[1] : "validate";
    if (mode == "validate") return validate();
    if (mode == "tensor") {
        const int bad = tensor_api<float>() + tensor_api<double>();
        std::printf("%s tensor (%d mismatches)\n", bad ? "FAILED" : "PASSED", bad);
        return bad ? 1 : 0;
    }
    int bad = 0;
    for (std::size_t r = 2; r <= 4; ++r) bad += kat_rank<float>(r) + kat_rank<double>(r);
    for (std::size_t k = 0; k < 6; ++k)
        if (pair_seen[k] == 0) {
            std::printf("slicing / fusion pair %zu never called\n", k);
            ++bad;
        }
    std::printf("%s kat (%d mismatches; %zu calls over 6 slicing/fusion pairs; %s)\n", bad ? "FAILED" : "PASSED",
                bad, pair_index, TLIBG_WITH_REFERENCE ? "reference headers" : "standalone");
    return bad ? 1 : 0;
}
