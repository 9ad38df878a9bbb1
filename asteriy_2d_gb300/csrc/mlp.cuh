// mlp.cuh - the learned start value of the exact Riemann solver.
//
// A 6-32-32-1 multilayer perceptron with SiLU activations predicts
// y = log(p*/p_L) for one face from
//   x = (rho_R/rho_L, p_R/p_L, (u_R - u_L)/c_L, c_R/c_L, gamma, log p_L)
// in the face frame (L = lower cell side, u = normal velocity).  The network
// first maps the three positive ratios to their logarithms and the velocity
// jump to its asinh (the raw ratios are heavy-tailed: thousands across
// strong shocks), then standardises each input with a shift and scale
// stored with the weights.  Parameter block (AST_MLP_NPARAM floats):
//   [0,6) shift  [6,12) scale  W1[32][6] at 12  b1[32] at 204
//   W2[32][32] at 236  b2[32] at 1260  w3[32] at 1292  b3 at 1324
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/asteriy_gb300.h"

namespace ast {

constexpr int kMlpIn = 6, kMlpH = 32;
constexpr int kOffShift = 0, kOffScale = 6, kOffW1 = 12, kOffB1 = 204, kOffW2 = 236, kOffB2 = 1260, kOffW3 = 1292,
              kOffB3 = 1324, kMlpParams = 1325;
static_assert(kMlpParams == AST_MLP_NPARAM, "parameter block size");

// The vectors of the block the tensor-core inference reads from shared
// memory (its W1 and W2 become mma fragments): shift, scale, b1, b2, w3, b3
constexpr int kVShift = 0, kVScale = 6, kVB1 = 12, kVB2 = 44, kVW3 = 76, kVB3 = 108, kVLen = 112;

// entry i of that compact vector block, from the parameter block W
__device__ __forceinline__ float mlp_vec(const float* W, int i)
{
    if (i < kVScale) return W[kOffShift + i];
    if (i < kVB1) return W[kOffScale + i - kVScale];
    if (i < kVB2) return W[kOffB1 + i - kVB1];
    if (i < kVW3) return W[kOffB2 + i - kVB2];
    if (i < kVB3) return W[kOffW3 + i - kVW3];
    return (i == kVB3) ? W[kOffB3] : 0.0f;
}

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

// the fixed input map: log of the positive ratios, asinh of the velocity jump
__device__ __forceinline__ float mlp_map(int i, float v)
{
    if (i == 0 || i == 1 || i == 3) return __logf(v);
    if (i == 2) return copysignf(__logf(fabsf(v) + sqrtf(v * v + 1.0f)), v);
    return v;
}

// forward pass; W may live in shared or global memory
__device__ __forceinline__ float mlp_forward(const float* __restrict__ W, const float xin[kMlpIn])
{
    float x[kMlpIn];
#pragma unroll
    for (int i = 0; i < kMlpIn; i++) x[i] = (mlp_map(i, xin[i]) - W[kOffShift + i]) * W[kOffScale + i];
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

// ------------------------------------------------------------------ tensor-core inference
// The same network evaluated for 16 faces at a time by one warp with
// mma.sync.m16n8k16 (f16 operands, f32 accumulation): layer 1 is one k-block
// (6 features padded to 16) times four n-tiles of 8 hidden units, layer 2 is
// two k-blocks times four n-tiles; the layer-1 accumulators are re-used in
// registers as layer 2's A operand (the m16n8 C fragments of n-tiles 2kb and
// 2kb+1 form the m16k16 A fragment of k-block kb).  SiLU(z) = h (1 + tanh h),
// h = z/2, with tanh.approx.f16x2.  B operands are pre-packed per lane.
namespace tc {

constexpr int kL1 = 4 * 32 * 2;          // packed words of W1: [n-tile][lane][reg]
constexpr int kL2 = 2 * 4 * 32 * 2;      // packed words of W2: [k-block][n-tile][lane][reg]

__device__ __forceinline__ unsigned pack_h2(float lo, float hi)
{
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<unsigned*>(&h);
}

__device__ __forceinline__ void mma16816(float c[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0,
                                         unsigned b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// SiLU of a pair of accumulators plus their biases, packed as f16x2
__device__ __forceinline__ unsigned silu_h2(float z0, float z1)
{
    __half2 h = __floats2half2_rn(0.5f * z0, 0.5f * z1);
    unsigned hu = *reinterpret_cast<unsigned*>(&h), t;
    asm("tanh.approx.f16x2 %0, %1;" : "=r"(t) : "r"(hu));
    __half2 th = *reinterpret_cast<__half2*>(&t);
    __half2 r = __hfma2(h, th, h);   // h * (1 + tanh h)
    return *reinterpret_cast<unsigned*>(&r);
}

// pack W1 and W2 of the float parameter block W into per-lane B fragments
__device__ __forceinline__ void pack_weights(const float* W, unsigned* B1, unsigned* B2)
{
    for (int i = threadIdx.x; i < kL1 + kL2; i += blockDim.x) {
        if (i < kL1) {
            const int j = i / 64, lane = (i / 2) % 32, reg = i % 2;
            const int g = lane >> 2, t = lane & 3, n = 8 * j + g, k = 2 * t + 8 * reg;
            const float w0 = (k < kMlpIn) ? W[kOffW1 + n * kMlpIn + k] : 0.0f;
            const float w1 = (k + 1 < kMlpIn) ? W[kOffW1 + n * kMlpIn + k + 1] : 0.0f;
            B1[i] = pack_h2(w0, w1);
        } else {
            const int q = i - kL1, kb = q / 256, j = (q / 64) % 4, lane = (q / 2) % 32, reg = q % 2;
            const int g = lane >> 2, t = lane & 3, n = 8 * j + g, k = 16 * kb + 2 * t + 8 * reg;
            B2[q] = pack_h2(W[kOffW2 + n * kMlpH + k], W[kOffW2 + n * kMlpH + k + 1]);
        }
    }
}

}  // namespace tc

// The packed network: the vector block (kVLen floats), then W1's and W2's
// B fragments (tc::kL1 + tc::kL2 words), in the order the step kernels hold
// them in shared memory, written once per upload after the parameter block
// of the device copy (at a 16-byte boundary), so that a tile copies it with
// 16-byte asynchronous copies instead of packing it
constexpr int kMlpPackOff = (kMlpParams + 3) / 4 * 4;
constexpr int kMlpPackWords = kVLen + tc::kL1 + tc::kL2;
constexpr int kMlpDevFloats = kMlpPackOff + kMlpPackWords;   // floats of the device copy
static_assert(kMlpPackWords % 4 == 0, "whole 16-byte copies");

// the packed network of the parameter block W into W + kMlpPackOff (all
// threads of one block)
__device__ __forceinline__ void pack_network(float* W)
{
    for (int i = threadIdx.x; i < kVLen; i += blockDim.x) W[kMlpPackOff + i] = mlp_vec(W, i);
    unsigned* B1 = reinterpret_cast<unsigned*>(W + kMlpPackOff + kVLen);
    tc::pack_weights(W, B1, B1 + tc::kL1);
}

namespace tc {

// y for 16 faces whose standardised features sit in X[16][8] (f32, cols 6-7
// zero); result for face r in y[r] (written by the lanes with t == 0).  V:
// the compact vector block (kV* offsets)
__device__ __forceinline__ void forward16(const float* V, const unsigned* B1, const unsigned* B2, const float (*X)[8],
                                          float* y)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const unsigned a0 = pack_h2(X[g][2 * t], X[g][2 * t + 1]);
    const unsigned a1 = pack_h2(X[g + 8][2 * t], X[g + 8][2 * t + 1]);
    // layer 1
    float c1[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float b0 = V[kVB1 + 8 * j + 2 * t], b1 = V[kVB1 + 8 * j + 2 * t + 1];
        c1[j][0] = b0; c1[j][1] = b1; c1[j][2] = b0; c1[j][3] = b1;
        mma16816(c1[j], a0, a1, 0u, 0u, B1[(j * 32 + lane) * 2], B1[(j * 32 + lane) * 2 + 1]);
    }
    unsigned h[4][2];   // SiLU(layer 1), f16x2: [n-tile][row g / g+8]
#pragma unroll
    for (int j = 0; j < 4; j++) {
        h[j][0] = silu_h2(c1[j][0], c1[j][1]);
        h[j][1] = silu_h2(c1[j][2], c1[j][3]);
    }
    // layer 2 and the output dot product
    float yg = 0.0f, yg8 = 0.0f;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const float b0 = V[kVB2 + 8 * j + 2 * t], b1 = V[kVB2 + 8 * j + 2 * t + 1];
        float c[4] = {b0, b1, b0, b1};
#pragma unroll
        for (int kb = 0; kb < 2; kb++) {
            const int idx = ((kb * 4 + j) * 32 + lane) * 2;
            mma16816(c, h[2 * kb][0], h[2 * kb][1], h[2 * kb + 1][0], h[2 * kb + 1][1], B2[idx], B2[idx + 1]);
        }
        const float w0 = V[kVW3 + 8 * j + 2 * t], w1 = V[kVW3 + 8 * j + 2 * t + 1];
        unsigned s0 = silu_h2(c[0], c[1]), s1 = silu_h2(c[2], c[3]);
        const float2 v0 = __half22float2(*reinterpret_cast<__half2*>(&s0));
        const float2 v1 = __half22float2(*reinterpret_cast<__half2*>(&s1));
        yg = fmaf(w0, v0.x, fmaf(w1, v0.y, yg));
        yg8 = fmaf(w0, v1.x, fmaf(w1, v1.y, yg8));
    }
    yg += __shfl_xor_sync(0xffffffffu, yg, 1);
    yg += __shfl_xor_sync(0xffffffffu, yg, 2);
    yg8 += __shfl_xor_sync(0xffffffffu, yg8, 1);
    yg8 += __shfl_xor_sync(0xffffffffu, yg8, 2);
    if (t == 0) {
        y[g] = yg + V[kVB3];
        y[g + 8] = yg8 + V[kVB3];
    }
}

}  // namespace tc

}  // namespace ast
