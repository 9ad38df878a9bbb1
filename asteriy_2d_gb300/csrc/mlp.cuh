// mlp.cuh - the learned start value of the exact Riemann solver.
//
// A 6-32-32-1 multilayer perceptron with SiLU activations predicts
// y = log(p*/p_L) for one face from
//   x = (rho_R/rho_L, p_R/p_L, (u_R - u_L)/c_L, c_R/c_L, gamma, log p_L)
// in the face frame (L = lower cell side, u = normal velocity).  The inputs
// are standardised with a per-feature shift and scale stored with the
// weights.  Parameter block (AST_MLP_NPARAM floats):
//   [0,6) shift  [6,12) scale  W1[32][6] at 12  b1[32] at 204
//   W2[32][32] at 236  b2[32] at 1260  w3[32] at 1292  b3 at 1324
#pragma once

#include <cuda_runtime.h>

#include "../../include/asteriy_gb300.h"

namespace ast {

constexpr int kMlpIn = 6, kMlpH = 32;
constexpr int kOffShift = 0, kOffScale = 6, kOffW1 = 12, kOffB1 = 204, kOffW2 = 236, kOffB2 = 1260, kOffW3 = 1292,
              kOffB3 = 1324, kMlpParams = 1325;
static_assert(kMlpParams == AST_MLP_NPARAM, "parameter block size");

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
// d silu / dz
__device__ __forceinline__ float silu_grad(float z)
{
    const float s = 1.0f / (1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// features of one face from its left/right states in the face frame
__device__ __forceinline__ void mlp_features(float gamma, float rL, float pL, float uL, float cL, float rR, float pR,
                                             float uR, float cR, float x[kMlpIn])
{
    x[0] = rR / rL;
    x[1] = pR / pL;
    x[2] = (uR - uL) / cL;
    x[3] = cR / cL;
    x[4] = gamma;
    x[5] = __logf(pL);
}

// forward pass; W may live in shared or global memory
__device__ __forceinline__ float mlp_forward(const float* __restrict__ W, const float xin[kMlpIn])
{
    float x[kMlpIn];
#pragma unroll
    for (int i = 0; i < kMlpIn; i++) x[i] = (xin[i] - W[kOffShift + i]) * W[kOffScale + i];
    float h1[kMlpH];
#pragma unroll
    for (int j = 0; j < kMlpH; j++) {
        float z = W[kOffB1 + j];
#pragma unroll
        for (int i = 0; i < kMlpIn; i++) z = fmaf(W[kOffW1 + j * kMlpIn + i], x[i], z);
        h1[j] = silu(z);
    }
    float y = W[kOffB3];
#pragma unroll 4
    for (int k = 0; k < kMlpH; k++) {
        float z = W[kOffB2 + k];
#pragma unroll
        for (int j = 0; j < kMlpH; j++) z = fmaf(W[kOffW2 + k * kMlpH + j], h1[j], z);
        y = fmaf(W[kOffW3 + k], silu(z), y);
    }
    return y;
}

}  // namespace ast
