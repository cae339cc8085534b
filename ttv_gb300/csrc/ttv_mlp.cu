// Training and inference kernels of the learned cost model (hand-written, fp32).
//
//   mlp_fwd_bwd   one thread per sample: forward pass, squared-error loss and
//                 the backward deltas of every layer (activations kept)
//   mlp_grad      one thread per parameter: the gradient summed over the
//                 minibatch in sample order (deterministic, no atomics)
//   mlp_adam      one thread per parameter: Adam update with bias correction
//   mlp_predict   one thread per row, weights staged in shared memory
//
// Loss: L = (1/n) sum_s 0.5 (f(x_s) - y_s)^2 over the minibatch.
#include "ttv_internal.h"
#include "ttv_mlp.cuh"

#include <map>
#include <mutex>
#include <vector>

namespace tlibg {

__global__ void __launch_bounds__(128) mlp_fwd_bwd(const float* __restrict__ w, const float* __restrict__ X,
                                                   const float* __restrict__ Y, const int* __restrict__ idx,
                                                   int n, float inv_n, float* Z1, float* Z2, float* Z3,
                                                   float* D1, float* D2, float* D3, float* Dout,
                                                   float* loss, float* Xb)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int row = idx ? idx[s] : s;
    float x[MLP_IN];
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) {
        x[i] = X[(size_t)row * MLP_IN + i];
        Xb[(size_t)s * MLP_IN + i] = x[i];
    }
    float* z1 = Z1 + (size_t)s * MLP_H;
    float* z2 = Z2 + (size_t)s * MLP_H;
    float* z3 = Z3 + (size_t)s * MLP_H;
    const float out = mlp_forward<true>(w, x, z1, z2, z3);
    const float err = out - Y[row];
    loss[s] = 0.5f * err * err * inv_n;
    const float dout = err * inv_n;
    Dout[s] = dout;
    float* d1 = D1 + (size_t)s * MLP_H;
    float* d2 = D2 + (size_t)s * MLP_H;
    float* d3 = D3 + (size_t)s * MLP_H;
    for (int j = 0; j < MLP_H; ++j) d3[j] = z3[j] > 0.f ? w[OFF_W4 + j] * dout : 0.f;
    for (int i = 0; i < MLP_H; ++i) {
        float acc = 0.f;
        if (z2[i] > 0.f)
            for (int j = 0; j < MLP_H; ++j) acc = fmaf(w[OFF_W3 + i * MLP_H + j], d3[j], acc);
        d2[i] = acc;
    }
    for (int i = 0; i < MLP_H; ++i) {
        float acc = 0.f;
        if (z1[i] > 0.f)
            for (int j = 0; j < MLP_H; ++j) acc = fmaf(w[OFF_W2 + i * MLP_H + j], d2[j], acc);
        d1[i] = acc;
    }
}

__device__ __forceinline__ float relu(float z) { return z > 0.f ? z : 0.f; }

__global__ void __launch_bounds__(128) mlp_grad(const float* __restrict__ Xb, const float* __restrict__ Z1,
                                                const float* __restrict__ Z2, const float* __restrict__ Z3,
                                                const float* __restrict__ D1, const float* __restrict__ D2,
                                                const float* __restrict__ D3, const float* __restrict__ Dout,
                                                int n, float* __restrict__ g)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= MLP_PARAMS) return;
    float acc = 0.f;
    if (p < OFF_B1) {
        const int i = p / MLP_H, j = p % MLP_H;
        for (int s = 0; s < n; ++s) acc = fmaf(Xb[(size_t)s * MLP_IN + i], D1[(size_t)s * MLP_H + j], acc);
    } else if (p < OFF_W2) {
        const int j = p - OFF_B1;
        for (int s = 0; s < n; ++s) acc += D1[(size_t)s * MLP_H + j];
    } else if (p < OFF_B2) {
        const int q = p - OFF_W2, i = q / MLP_H, j = q % MLP_H;
        for (int s = 0; s < n; ++s) acc = fmaf(relu(Z1[(size_t)s * MLP_H + i]), D2[(size_t)s * MLP_H + j], acc);
    } else if (p < OFF_W3) {
        const int j = p - OFF_B2;
        for (int s = 0; s < n; ++s) acc += D2[(size_t)s * MLP_H + j];
    } else if (p < OFF_B3) {
        const int q = p - OFF_W3, i = q / MLP_H, j = q % MLP_H;
        for (int s = 0; s < n; ++s) acc = fmaf(relu(Z2[(size_t)s * MLP_H + i]), D3[(size_t)s * MLP_H + j], acc);
    } else if (p < OFF_W4) {
        const int j = p - OFF_B3;
        for (int s = 0; s < n; ++s) acc += D3[(size_t)s * MLP_H + j];
    } else if (p < OFF_B4) {
        const int j = p - OFF_W4;
        for (int s = 0; s < n; ++s) acc = fmaf(relu(Z3[(size_t)s * MLP_H + j]), Dout[s], acc);
    } else {
        for (int s = 0; s < n; ++s) acc += Dout[s];
    }
    g[p] = acc;
}

// Sum of the per-sample losses in a fixed tree order (one CTA of 256).
__global__ void __launch_bounds__(256) mlp_loss_sum(const float* __restrict__ loss, int n, float* out, int accumulate)
{
    __shared__ float sh[256];
    float acc = 0.f;
    for (int s = threadIdx.x; s < n; s += 256) acc += loss[s];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int off = 128; off > 0; off >>= 1) {
        if (threadIdx.x < off) sh[threadIdx.x] += sh[threadIdx.x + off];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = accumulate ? out[0] + sh[0] : sh[0];
}

__global__ void __launch_bounds__(256) mlp_adam(float* __restrict__ w, const float* __restrict__ g,
                                                float* __restrict__ m, float* __restrict__ v, int np,
                                                float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const float gp = g[p];
    const float mp = b1 * m[p] + (1.f - b1) * gp;
    const float vp = b2 * v[p] + (1.f - b2) * gp * gp;
    m[p] = mp;
    v[p] = vp;
    w[p] -= lr * (mp / c1) / (sqrtf(vp / c2) + eps);
}

__global__ void __launch_bounds__(128) mlp_predict(const float* __restrict__ w, const float* __restrict__ X,
                                                   int n, float* __restrict__ Y)
{
    __shared__ float sw[MLP_PARAMS];
    for (int p = threadIdx.x; p < MLP_PARAMS; p += blockDim.x) sw[p] = w[p];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float x[MLP_IN];
#pragma unroll
    for (int i = 0; i < MLP_IN; ++i) x[i] = X[(size_t)s * MLP_IN + i];
    Y[s] = mlp_forward<false>(sw, x, nullptr, nullptr, nullptr);
}

namespace {

// per-(device, stream) workspace of the training kernels, grow-only
struct Work {
    float* buf = nullptr;
    size_t rows = 0;
    int* idx = nullptr;
    size_t idx_n = 0;
};
std::mutex g_mu;
std::map<std::pair<int, uintptr_t>, Work> g_work;

int workspace(cudaStream_t st, size_t rows, Work** out)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_mu);
    Work& w = g_work[{dev, reinterpret_cast<uintptr_t>(st)}];
    if (w.rows < rows) {
        if (w.buf) {
            cudaStreamSynchronize(st);
            cudaFree(w.buf);
        }
        w.buf = nullptr;
        w.rows = 0;
        const size_t floats = rows * (6 * MLP_H + MLP_IN + 2) + 4;
        cudaError_t e = internal_malloc((void**)&w.buf, floats * sizeof(float));
        if (e != cudaSuccess) return internal_cuda_fail(e, "cost-model workspace");
        w.rows = rows;
    }
    *out = &w;
    return TLIBG_OK;
}

int loss_grad(const float* params, const float* x, const float* y, const int* idx, size_t n,
              float* grad, float* loss, int accumulate, cudaStream_t st)
{
    Work* w = nullptr;
    int s = workspace(st, n, &w);
    if (s) return s;
    float* Z1 = w->buf;
    float* Z2 = Z1 + n * MLP_H;
    float* Z3 = Z2 + n * MLP_H;
    float* D1 = Z3 + n * MLP_H;
    float* D2 = D1 + n * MLP_H;
    float* D3 = D2 + n * MLP_H;
    float* Xb = D3 + n * MLP_H;
    float* Dout = Xb + n * MLP_IN;
    float* L = Dout + n;
    const int blocks = (int)((n + 127) / 128);
    mlp_fwd_bwd<<<blocks, 128, 0, st>>>(params, x, y, idx, (int)n, 1.f / (float)n, Z1, Z2, Z3, D1, D2,
                                        D3, Dout, L, Xb);
    mlp_grad<<<(MLP_PARAMS + 127) / 128, 128, 0, st>>>(Xb, Z1, Z2, Z3, D1, D2, D3, Dout, (int)n, grad);
    mlp_loss_sum<<<1, 256, 0, st>>>(L, (int)n, loss, accumulate);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return internal_cuda_fail(e, "cost-model kernels");
    internal_count_launches(3);
    return TLIBG_OK;
}

}  // namespace
}  // namespace tlibg

using namespace tlibg;

extern "C" {

int tlibg_mlp_loss_grad(const float* params, const float* x, const float* y, size_t n, float* grad,
                        float* loss, void* stream)
{
    if (!params || !x || !y || !grad || !loss || n == 0)
        return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_mlp_loss_grad: null buffer or empty batch");
    int s = loss_grad(params, x, y, nullptr, n, grad, loss, 0, static_cast<cudaStream_t>(stream));
    return s ? s : internal_ok();
}

int tlibg_mlp_adam(float* params, const float* grad, float* m, float* v, uint64_t step, float lr,
                   float beta1, float beta2, float eps, void* stream)
{
    if (!params || !grad || !m || !v || step == 0)
        return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_mlp_adam: null buffer or step 0");
    const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
    mlp_adam<<<(MLP_PARAMS + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        params, grad, m, v, MLP_PARAMS, lr, beta1, beta2, eps, c1, c2);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return internal_cuda_fail(e, "mlp_adam");
    internal_count_launches(1);
    return internal_ok();
}

int tlibg_mlp_predict(const float* params, const float* x, size_t n, float* y, void* stream)
{
    if (!params || !x || !y) return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_mlp_predict: null buffer");
    if (n == 0) return internal_ok();
    mlp_predict<<<(int)((n + 127) / 128), 128, 0, static_cast<cudaStream_t>(stream)>>>(params, x, (int)n, y);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return internal_cuda_fail(e, "mlp_predict");
    internal_count_launches(1);
    return internal_ok();
}

int tlibg_mlp_train(float* params, float* m, float* v, const float* x, const float* y, size_t n,
                    int epochs, int batch, float lr, uint64_t seed, float* epoch_loss, void* stream)
{
    if (!params || !m || !v || !x || !y || n == 0 || epochs <= 0 || batch <= 0)
        return internal_fail(TLIBG_ERR_ARGUMENT, "tlibg_mlp_train: bad arguments");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *grad = nullptr, *loss = nullptr;
    int* idx = nullptr;
    cudaError_t e;
    if ((e = internal_malloc((void**)&grad, MLP_PARAMS * sizeof(float))) != cudaSuccess) return internal_cuda_fail(e, "train grad");
    if ((e = internal_malloc((void**)&loss, sizeof(float))) != cudaSuccess) return internal_cuda_fail(e, "train loss");
    if ((e = internal_malloc((void**)&idx, n * sizeof(int))) != cudaSuccess) return internal_cuda_fail(e, "train idx");
    std::vector<int> perm(n);
    uint64_t state = seed * 6364136223846793005ull + 1442695040888963407ull;
    auto next = [&state]() {
        state ^= state << 13;
        state ^= state >> 7;
        state ^= state << 17;
        return state;
    };
    uint64_t step = 0;
    int status = TLIBG_OK;
    for (int ep = 0; ep < epochs && !status; ++ep) {
        for (size_t i = 0; i < n; ++i) perm[i] = (int)i;
        for (size_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[next() % (i + 1)]);
        cudaMemcpyAsync(idx, perm.data(), n * sizeof(int), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(loss, 0, sizeof(float), st);
        for (size_t b0 = 0; b0 < n && !status; b0 += batch) {
            const size_t nb = std::min<size_t>(batch, n - b0);
            status = loss_grad(params, x, y, idx + b0, nb, grad, loss, 1, st);
            if (status) break;
            ++step;
            const float c1 = 1.f - powf(0.9f, (float)step), c2 = 1.f - powf(0.999f, (float)step);
            mlp_adam<<<(MLP_PARAMS + 255) / 256, 256, 0, st>>>(params, grad, m, v, MLP_PARAMS, lr, 0.9f,
                                                               0.999f, 1e-8f, c1, c2);
            internal_count_launches(1);
        }
        if (epoch_loss) {
            float h = 0.f;
            cudaMemcpyAsync(&h, loss, sizeof(float), cudaMemcpyDeviceToHost, st);
            cudaStreamSynchronize(st);
            // minibatch losses are means; report the epoch mean
            epoch_loss[ep] = h * (float)batch / (float)n;
        }
    }
    e = cudaStreamSynchronize(st);
    cudaFree(grad);
    cudaFree(loss);
    cudaFree(idx);
    if (status) return status;
    if (e != cudaSuccess) return internal_cuda_fail(e, "train synchronize");
    return internal_ok();
}

}  // extern "C"
