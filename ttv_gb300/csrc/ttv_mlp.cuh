// Learned cost model shared by the training kernels (ttv_mlp.cu) and the
// variant-selection kernel of the batched launch (ttv_batch.cu).
//
// A multilayer perceptron with three hidden layers of 64 ReLU units that maps
// (problem features, one-hot variant) to the predicted log2 of the variant's
// cost per problem in microseconds.  Parameters are one flat float array:
//   W1[IN][H]  b1[H]  W2[H][H]  b2[H]  W3[H][H]  b3[H]  W4[H]  b4
#pragma once

#include <stdint.h>

namespace tlibg {

constexpr int NFEAT = 8;      // shape features of a problem (see batch_features)
constexpr int NVARIANT = 9;   // kernel variants a batched problem can run with
constexpr int MLP_IN = NFEAT + NVARIANT;
constexpr int MLP_H = 64;
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + MLP_IN * MLP_H;
constexpr int OFF_W2 = OFF_B1 + MLP_H;
constexpr int OFF_B2 = OFF_W2 + MLP_H * MLP_H;
constexpr int OFF_W3 = OFF_B2 + MLP_H;
constexpr int OFF_B3 = OFF_W3 + MLP_H * MLP_H;
constexpr int OFF_W4 = OFF_B3 + MLP_H;
constexpr int OFF_B4 = OFF_W4 + MLP_H;
constexpr int MLP_PARAMS = OFF_B4 + 1;

// Forward pass of one input row; keeps the activations when `keep` is set
// (training).  `w` may point to global or shared memory.
template <bool KEEP>
__device__ __forceinline__ float mlp_forward(const float* __restrict__ w, const float* x, float* a1,
                                             float* a2, float* a3)
{
    float h1[MLP_H], h2[MLP_H];
#pragma unroll 4
    for (int j = 0; j < MLP_H; ++j) {
        float z = w[OFF_B1 + j];
#pragma unroll
        for (int i = 0; i < MLP_IN; ++i) z = fmaf(x[i], w[OFF_W1 + i * MLP_H + j], z);
        h1[j] = z > 0.f ? z : 0.f;
        if (KEEP) a1[j] = z;
    }
#pragma unroll 4
    for (int j = 0; j < MLP_H; ++j) {
        float z = w[OFF_B2 + j];
#pragma unroll
        for (int i = 0; i < MLP_H; ++i) z = fmaf(h1[i], w[OFF_W2 + i * MLP_H + j], z);
        h2[j] = z > 0.f ? z : 0.f;
        if (KEEP) a2[j] = z;
    }
    float out = w[OFF_B4];
#pragma unroll 4
    for (int j = 0; j < MLP_H; ++j) {
        float z = w[OFF_B3 + j];
#pragma unroll
        for (int i = 0; i < MLP_H; ++i) z = fmaf(h2[i], w[OFF_W3 + i * MLP_H + j], z);
        if (KEEP) a3[j] = z;
        out = fmaf(z > 0.f ? z : 0.f, w[OFF_W4 + j], out);
    }
    return out;
}

}  // namespace tlibg
