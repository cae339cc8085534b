/*
 * tlib/ttv_gpu_tensor.h -- device-resident tensor with tlib's high-level
 * tensor-times-vector interface.
 *
 * Mirrors the reference's tensor<T> / tensor_view<T> (include/tlib/detail/
 * tensor.h:36-114), its high-level ttv(q, A, b, ...) (include/tlib/ttv.h:
 * 98-114) and A(q) * b (ttv.h:122-127), with the data in device memory:
 *
 *     tlib::ttv::gpu::tensor<float> A({256, 256, 256}, {1, 2, 3});
 *     tlib::ttv::gpu::tensor<float> b({256});
 *     A.from_host(a_values);  b = 1.0f;
 *     auto C = A(2) * b;                    // computed on the GPU, stays there
 *     std::vector<float> c = C.to_host();
 *
 * Same checks and exception texts as the reference's tensor constructor and
 * call operator; C's shape and layout follow the reference's rules
 * (shape.h:103-158, layout.h:143-207).  With the reference headers on the
 * include path, a device tensor can be made from / turned into the
 * reference's host tensor<T>.  Move-only; the destructor frees the memory.
 */
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <numeric>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "ttv_gpu.h"

namespace tlib::ttv::gpu {

template <class value_t> class tensor;

namespace tensor_detail {

inline void cuda_check(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw std::runtime_error(std::string("tlibg: ") + what + ": " + cudaGetErrorString(e));
}

inline bool valid_shape(const std::vector<std::size_t>& n)
{
    return !n.empty() && std::none_of(n.begin(), n.end(), [](std::size_t a) { return a == 0u; });
}

inline bool valid_layout(const std::vector<std::size_t>& pi)
{
    const std::size_t n = pi.size();
    if (n == 0) return false;
    for (std::size_t i = 0; i < n; ++i) {
        if (pi[i] == 0u || pi[i] > n) return false;
        if (std::find(pi.begin() + i + 1, pi.end(), pi[i]) != pi.end()) return false;
    }
    return true;
}

inline std::vector<std::size_t> first_order(std::size_t p)
{
    std::vector<std::size_t> pi(p);
    std::iota(pi.begin(), pi.end(), std::size_t(1));
    return pi;
}

}  // namespace tensor_detail

template <class _value_t> struct tensor_view {
  public:
    using value_t = _value_t;
    using tensor_t = tensor<value_t>;
    tensor_view() = delete;
    tensor_view(tensor_view const&) = delete;
    tensor_view& operator=(tensor_view const&) = delete;
    tensor_t const& get_tensor() const { return _tensor; }
    std::size_t contraction_mode() const { return _q; }

  private:
    friend class tensor<value_t>;
    tensor_view(tensor_t const& t, std::size_t q) : _tensor(t), _q(q) {}
    tensor_t const& _tensor;
    std::size_t _q;
};

template <class value_t> class tensor {
  public:
    using shape_t = std::vector<std::size_t>;
    using layout_t = std::vector<std::size_t>;
    using strides_t = std::vector<std::size_t>;
    using tensor_view_t = tensor_view<value_t>;

    tensor() = delete;

    // Uninitialised device storage for a dense tensor of shape n and layout pi.
    tensor(shape_t const& n, layout_t const& pi) : _n(n), _pi(pi)
    {
        if (n.size() != pi.size())
            throw std::runtime_error("Error in tlib::tensor: shape vector and layout vector must have the same length.");
        if (!tensor_detail::valid_shape(n))
            throw std::runtime_error("Error in tlib::tensor: shape vector of tensor is not valid.");
        if (!tensor_detail::valid_layout(pi))
            throw std::runtime_error("Error in tlib::tensor: layout vector of tensor is not valid.");
        _size = std::accumulate(n.begin(), n.end(), std::size_t(1), std::multiplies<>());
        void* p = nullptr;
        tensor_detail::cuda_check(cudaMalloc(&p, _size * sizeof(value_t)), "cudaMalloc");
        _data = static_cast<value_t*>(p);
    }

    explicit tensor(shape_t const& n) : tensor(n, tensor_detail::first_order(n.size())) {}

    tensor(shape_t const& n, layout_t const& pi, std::vector<value_t> const& host) : tensor(n, pi)
    {
        from_host(host);
    }

#if TLIBG_WITH_REFERENCE
    // Upload one of the reference's host tensors (same shape and layout).
    explicit tensor(tlib::ttv::tensor<value_t> const& h) : tensor(h.shape(), h.layout(), h.data()) {}

    // Download into one of the reference's host tensors.
    tlib::ttv::tensor<value_t> host() const
    {
        tlib::ttv::tensor<value_t> h(_n, _pi);
        tensor_detail::cuda_check(cudaMemcpy(h.data().data(), _data, _size * sizeof(value_t), cudaMemcpyDeviceToHost),
                                  "cudaMemcpy");
        return h;
    }
#endif

    tensor(tensor const&) = delete;
    tensor& operator=(tensor const&) = delete;
    tensor(tensor&& o) noexcept : _n(std::move(o._n)), _pi(std::move(o._pi)), _size(o._size), _data(o._data)
    {
        o._data = nullptr;
        o._size = 0;
    }
    tensor& operator=(tensor&& o) noexcept
    {
        if (this != &o) {
            release();
            _n = std::move(o._n);
            _pi = std::move(o._pi);
            _size = o._size;
            _data = o._data;
            o._data = nullptr;
            o._size = 0;
        }
        return *this;
    }
    ~tensor() { release(); }

    // Every element set to v (on the device).
    tensor& operator=(value_t v)
    {
        if (v == value_t(0)) {
            tensor_detail::cuda_check(cudaMemset(_data, 0, _size * sizeof(value_t)), "cudaMemset");
        } else {
            std::vector<value_t> h(_size, v);
            from_host(h);
        }
        return *this;
    }

    tensor_view_t operator()(std::size_t contraction_mode) const
    {
        if (1ul > contraction_mode || contraction_mode > this->order())
            throw std::runtime_error("Error in tlib::tensor: specified contraction mode should be greater than one "
                                     "and equal to or less than the order.");
        return tensor_view_t(*this, contraction_mode);
    }

    void from_host(std::vector<value_t> const& h)
    {
        if (h.size() != _size) throw std::runtime_error("tlibg: host data does not match the tensor's size");
        tensor_detail::cuda_check(cudaMemcpy(_data, h.data(), _size * sizeof(value_t), cudaMemcpyHostToDevice),
                                  "cudaMemcpy");
    }

    std::vector<value_t> to_host() const
    {
        std::vector<value_t> h(_size);
        tensor_detail::cuda_check(cudaMemcpy(h.data(), _data, _size * sizeof(value_t), cudaMemcpyDeviceToHost),
                                  "cudaMemcpy");
        return h;
    }

    value_t* data() { return _data; }
    const value_t* data() const { return _data; }
    shape_t const& shape() const { return _n; }
    layout_t const& layout() const { return _pi; }
    strides_t strides() const
    {
        strides_t w(_n.size());
        gpu_detail::throw_status(tlibg_strides(_n.data(), _pi.data(), _n.size(), w.data()));
        return w;
    }
    std::size_t order() const { return _n.size(); }
    std::size_t size() const { return _size; }

  private:
    void release()
    {
        if (_data) cudaFree(_data);
        _data = nullptr;
    }
    shape_t _n;
    layout_t _pi;
    std::size_t _size = 0;
    value_t* _data = nullptr;
};

// C = A x_q b on the device (reference ttv.h:98-114): C gets the shape and
// layout the reference derives from A's; returns when C is complete, or
// enqueues on `stream` when one is given (C's storage then belongs to the
// caller's stream order).
template <class value_t>
inline tensor<value_t> ttv(std::size_t q, tensor<value_t> const& a, tensor<value_t> const& b, void* stream = nullptr)
{
    const std::size_t p = a.order();
    if (q == 0 || q > p)
        throw std::runtime_error("Error in tlib::tensor_times_vector: contraction mode should be greater zero or less "
                                 "than or equal to p.");
    std::vector<std::size_t> nc(p > 1 ? p - 1 : 1), pic(p > 1 ? p - 1 : 1);
    gpu_detail::throw_status(tlibg_output_shape(a.shape().data(), p, q, nc.data()));
    gpu_detail::throw_status(tlibg_output_layout(a.layout().data(), p, q, pic.data()));
    tensor<value_t> c(nc, pic);
    const auto wa = a.strides();
    const auto wc = c.strides();
    if (stream)
        tlib::ttv::ttv(execution_policy::gpu_on(stream), slicing_policy::subtensor, fusion_policy::all, q, p, a.data(),
                       a.shape().data(), wa.data(), a.layout().data(), b.data(), b.shape().data(), c.data(),
                       c.shape().data(), wc.data(), c.layout().data());
    else
        tlib::ttv::ttv(execution_policy::gpu, slicing_policy::subtensor, fusion_policy::all, q, p, a.data(),
                       a.shape().data(), wa.data(), a.layout().data(), b.data(), b.shape().data(), c.data(),
                       c.shape().data(), wc.data(), c.layout().data());
    return c;
}

// A(q) * b (reference ttv.h:122-127), on the device.
template <class value_t> inline tensor<value_t> operator*(tensor_view<value_t> const& a, tensor<value_t> const& b)
{
    return ttv(a.contraction_mode(), a.get_tensor(), b);
}

}  // namespace tlib::ttv::gpu
