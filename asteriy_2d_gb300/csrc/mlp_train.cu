// mlp_train.cu - forward, backward and Adam kernels of the learned start
// value (the network of mlp.cuh), and the C entry points that train it.
//
// Loss: mean squared error of y = log(p*/p_L) over a batch.  One thread
// carries one sample through the forward and backward pass; the CTA then
// reduces the per-sample weight gradients from shared memory (each weight
// gradient is a sum over the CTA's samples of an outer-product term) and
// adds its partial gradient to the global one with atomics.  The network is
// too small (1313 weights) for tensor-core tiles to pay; everything is FP32
// SIMT.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/asteriy_gb300.h"
#include "mlp.cuh"

namespace ast {
int cuda_fail(cudaError_t e, const char* what);
}

using namespace ast;

namespace {

constexpr int kB = 256;          // samples per CTA
constexpr int kH = kMlpH, kI = kMlpIn;
constexpr int kPad = kH + 1;     // row pitch of the per-sample activations (no bank conflicts)

struct GradSmem {
    float W[kMlpParams];
    float X[kB][kI];
    float H1[kB][kPad];
    float H2[kB][kPad];
    float DZ1[kB][kPad];
    float DZ2[kB][kPad];
    float DY[kB];
};

// samples: n records of AST_RECORD_FLOATS (x[6], target, ...); idx: optional
// permutation (sample i of this pass is samples[idx[i]]).  grad (1325 floats,
// the shift/scale slots stay zero) and loss_sum are accumulated.
__global__ void __launch_bounds__(kB) mlp_grad_kernel(const float* __restrict__ W_g, const float* __restrict__ samples,
                                                      const int* __restrict__ idx, long long first, long long count,
                                                      float inv_count, float* __restrict__ grad, float* loss_sum)
{
    extern __shared__ __align__(16) unsigned char raw[];
    GradSmem& s = *reinterpret_cast<GradSmem*>(raw);
    const int t = threadIdx.x;
    for (int i = t; i < kMlpParams; i += kB) s.W[i] = W_g[i];
    __syncthreads();

    const long long gi = (long long)blockIdx.x * kB + t;
    const bool valid = gi < count;
    float x[kI], target = 0.0f;
    if (valid) {
        const long long k = idx ? (long long)idx[first + gi] : first + gi;
        const float* r = samples + k * AST_RECORD_FLOATS;
#pragma unroll
        for (int i = 0; i < kI; i++) x[i] = (mlp_map(i, r[i]) - s.W[kOffShift + i]) * s.W[kOffScale + i];
        target = r[6];
    } else {
#pragma unroll
        for (int i = 0; i < kI; i++) x[i] = 0.0f;
    }
    // forward
    float z1[kH], h1[kH];
#pragma unroll
    for (int j = 0; j < kH; j++) {
        float z = s.W[kOffB1 + j];
#pragma unroll
        for (int i = 0; i < kI; i++) z = fmaf(s.W[kOffW1 + j * kI + i], x[i], z);
        z1[j] = z;
        h1[j] = silu(z);
    }
    float y = s.W[kOffB3];
    float z2[kH];
#pragma unroll 4
    for (int k = 0; k < kH; k++) {
        float z = s.W[kOffB2 + k];
#pragma unroll
        for (int j = 0; j < kH; j++) z = fmaf(s.W[kOffW2 + k * kH + j], h1[j], z);
        z2[k] = z;
        y = fmaf(s.W[kOffW3 + k], silu(z), y);
    }
    const float err = valid ? (y - target) : 0.0f;
    const float dy = 2.0f * err * inv_count;
    // backward through the output and the second layer
    float dh1[kH];
#pragma unroll
    for (int j = 0; j < kH; j++) dh1[j] = 0.0f;
#pragma unroll 4
    for (int k = 0; k < kH; k++) {
        const float h2 = silu(z2[k]);
        const float dz2 = dy * s.W[kOffW3 + k] * silu_grad(z2[k]);
        s.H2[t][k] = h2;
        s.DZ2[t][k] = dz2;
#pragma unroll
        for (int j = 0; j < kH; j++) dh1[j] = fmaf(s.W[kOffW2 + k * kH + j], dz2, dh1[j]);
    }
#pragma unroll
    for (int j = 0; j < kH; j++) {
        s.H1[t][j] = h1[j];
        s.DZ1[t][j] = dh1[j] * silu_grad(z1[j]);
    }
#pragma unroll
    for (int i = 0; i < kI; i++) s.X[t][i] = x[i];
    s.DY[t] = dy;
    // loss
    float l = err * err;
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((t & 31) == 0 && l != 0.0f) atomicAdd(loss_sum, l);
    __syncthreads();

    // CTA reduction over samples of the outer-product gradient terms
    for (int o = t; o < kH * kH; o += kB) {           // W2[k][j]: sum_s dz2[s][k] h1[s][j]
        const int k = o / kH, j = o - k * kH;
        float acc = 0.0f;
        for (int q = 0; q < kB; q++) acc = fmaf(s.DZ2[q][k], s.H1[q][j], acc);
        if (acc != 0.0f) atomicAdd(&grad[kOffW2 + o], acc);
    }
    for (int o = t; o < kH * kI + 3 * kH + 1; o += kB) {
        float acc = 0.0f;
        int dst;
        if (o < kH * kI) {                             // W1[j][i]: sum_s dz1[s][j] x[s][i]
            const int j = o / kI, i = o - j * kI;
            for (int q = 0; q < kB; q++) acc = fmaf(s.DZ1[q][j], s.X[q][i], acc);
            dst = kOffW1 + o;
        } else if (o < kH * kI + kH) {                 // b1[j]
            const int j = o - kH * kI;
            for (int q = 0; q < kB; q++) acc += s.DZ1[q][j];
            dst = kOffB1 + j;
        } else if (o < kH * kI + 2 * kH) {             // b2[k]
            const int k = o - kH * kI - kH;
            for (int q = 0; q < kB; q++) acc += s.DZ2[q][k];
            dst = kOffB2 + k;
        } else if (o < kH * kI + 3 * kH) {             // w3[k]: sum_s dy[s] h2[s][k]
            const int k = o - kH * kI - 2 * kH;
            for (int q = 0; q < kB; q++) acc = fmaf(s.DY[q], s.H2[q][k], acc);
            dst = kOffW3 + k;
        } else {                                       // b3
            for (int q = 0; q < kB; q++) acc += s.DY[q];
            dst = kOffB3;
        }
        if (acc != 0.0f) atomicAdd(&grad[dst], acc);
    }
}

// Adam step on the trainable slots (shift/scale are fixed); zeroes grad
__global__ void adam_kernel(float* __restrict__ W, float* __restrict__ grad, float* __restrict__ m1,
                            float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kOffW1 || i >= kMlpParams) return;
    const float gr = grad[i];
    grad[i] = 0.0f;
    const float a = b1 * m1[i] + (1.0f - b1) * gr;
    const float v = b2 * m2[i] + (1.0f - b2) * gr * gr;
    m1[i] = a;
    m2[i] = v;
    W[i] -= lr * (a * c1) / (sqrtf(v * c2) + eps);
}

__global__ void mlp_forward_kernel(const float* __restrict__ W_g, const float* __restrict__ x, long long n,
                                   int stride, float* __restrict__ y)
{
    __shared__ float W[kMlpParams];
    for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) W[i] = W_g[i];
    __syncthreads();
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    float xin[kI];
#pragma unroll
    for (int i = 0; i < kI; i++) xin[i] = x[k * stride + i];
    y[k] = mlp_forward(W, xin);
}

thread_local std::string g_err;

struct DevBuf {
    void* p = nullptr;
    ~DevBuf() { cudaFree(p); }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes); }
    template <typename T> T* as() { return (T*)p; }
};

#define TRY(call)                                                   \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return ast::cuda_fail(e_, #call);    \
    } while (0)

int set_grad_smem()
{
    static bool done = false;
    if (!done) {
        TRY(cudaFuncSetAttribute(mlp_grad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(GradSmem)));
        done = true;
    }
    return AST_OK;
}

}  // namespace

extern "C" {

// Initial parameters: input shift/scale = mean and 1/std of the samples'
// mapped features (log of the positive ratios, asinh of the velocity jump),
// weights ~ U(-sqrt(6/(fan_in+fan_out)), +...) from mt19937_64(seed),
// biases 0, output bias = mean target.  Host function.
int ast_mlp_init(const float* samples, int64_t n, uint64_t seed, float* params)
{
    if (!samples || !params || n < 2) return AST_ERR_INVALID;
    std::memset(params, 0, sizeof(float) * AST_MLP_NPARAM);
    double mean[kI] = {0}, sq[kI] = {0}, ty = 0.0;
    for (int64_t k = 0; k < n; k++) {
        const float* r = samples + k * AST_RECORD_FLOATS;
        for (int i = 0; i < kI; i++) {
            double v = r[i];
            if (i == 0 || i == 1 || i == 3) v = std::log(v);
            else if (i == 2) v = std::asinh(v);
            mean[i] += v;
            sq[i] += v * v;
        }
        ty += r[6];
    }
    for (int i = 0; i < kI; i++) {
        const double m = mean[i] / n;
        const double var = std::max(sq[i] / n - m * m, 0.0);
        params[kOffShift + i] = (float)m;
        params[kOffScale + i] = (float)(var > 1e-12 ? 1.0 / std::sqrt(var) : 1.0);
    }
    std::mt19937_64 gen(seed);
    auto uni = [&](double lim) { return (float)(((gen() >> 11) * 0x1.0p-53 * 2.0 - 1.0) * lim); };
    const double l1 = std::sqrt(6.0 / (kI + kH)), l2 = std::sqrt(6.0 / (kH + kH)), l3 = std::sqrt(6.0 / (kH + 1));
    for (int i = 0; i < kH * kI; i++) params[kOffW1 + i] = uni(l1);
    for (int i = 0; i < kH * kH; i++) params[kOffW2 + i] = uni(l2);
    for (int i = 0; i < kH; i++) params[kOffW3 + i] = uni(l3);
    params[kOffB3] = (float)(ty / n);
    return AST_OK;
}

// Mean-squared-error loss and its gradient over n host samples (device
// kernels).  grad: AST_MLP_NPARAM floats (shift/scale slots 0).
int ast_mlp_grad(const float* params, const float* samples, int64_t n, float* grad, float* loss)
{
    if (!params || !samples || !grad || n < 1) return AST_ERR_INVALID;
    int rc = set_grad_smem();
    if (rc != AST_OK) return rc;
    DevBuf dW, dS, dG, dL;
    TRY(dW.alloc(sizeof(float) * kMlpParams));
    TRY(dS.alloc(sizeof(float) * AST_RECORD_FLOATS * n));
    TRY(dG.alloc(sizeof(float) * kMlpParams));
    TRY(dL.alloc(sizeof(float)));
    TRY(cudaMemcpy(dW.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(dS.p, samples, sizeof(float) * AST_RECORD_FLOATS * n, cudaMemcpyHostToDevice));
    TRY(cudaMemset(dG.p, 0, sizeof(float) * kMlpParams));
    TRY(cudaMemset(dL.p, 0, sizeof(float)));
    const int blocks = (int)((n + kB - 1) / kB);
    mlp_grad_kernel<<<blocks, kB, sizeof(GradSmem)>>>(dW.as<float>(), dS.as<float>(), nullptr, 0, n, 1.0f / (float)n,
                                                       dG.as<float>(), dL.as<float>());
    TRY(cudaGetLastError());
    TRY(cudaMemcpy(grad, dG.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    float l = 0.0f;
    TRY(cudaMemcpy(&l, dL.p, sizeof(float), cudaMemcpyDeviceToHost));
    if (loss) *loss = l / (float)n;
    return AST_OK;
}

int ast_mlp_forward(const float* params, const float* x, int64_t n, int stride, float* y)
{
    if (!params || !x || !y || n < 1 || stride < kI) return AST_ERR_INVALID;
    DevBuf dW, dX, dY;
    TRY(dW.alloc(sizeof(float) * kMlpParams));
    TRY(dX.alloc(sizeof(float) * stride * n));
    TRY(dY.alloc(sizeof(float) * n));
    TRY(cudaMemcpy(dW.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(dX.p, x, sizeof(float) * stride * n, cudaMemcpyHostToDevice));
    mlp_forward_kernel<<<(int)((n + 255) / 256), 256>>>(dW.as<float>(), dX.as<float>(), n, stride, dY.as<float>());
    TRY(cudaGetLastError());
    TRY(cudaMemcpy(y, dY.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return AST_OK;
}

// Adam on the GPU: `epochs` passes over the n host samples in batches of
// `batch` (a multiple of 256), the sample order drawn once from
// mt19937_64(seed) and the batch order redrawn every epoch.  params holds the
// initial parameters (ast_mlp_init) and receives the trained ones;
// loss_per_epoch (optional, `epochs` floats) the mean batch loss.
int ast_mlp_train(const float* samples, int64_t n, int epochs, int batch, float lr, uint64_t seed, float* params,
                  float* loss_per_epoch)
{
    if (!samples || !params || n < batch || epochs < 1 || batch < kB || batch % kB) return AST_ERR_INVALID;
    int rc = set_grad_smem();
    if (rc != AST_OK) return rc;
    const int64_t nb = n / batch;
    std::vector<int> perm(n);
    for (int64_t i = 0; i < n; i++) perm[i] = (int)i;
    std::mt19937_64 gen(seed);
    std::shuffle(perm.begin(), perm.end(), gen);
    DevBuf dW, dS, dG, dM1, dM2, dL, dI;
    TRY(dW.alloc(sizeof(float) * kMlpParams));
    TRY(dS.alloc(sizeof(float) * AST_RECORD_FLOATS * n));
    TRY(dI.alloc(sizeof(int) * n));
    TRY(dG.alloc(sizeof(float) * kMlpParams));
    TRY(dM1.alloc(sizeof(float) * kMlpParams));
    TRY(dM2.alloc(sizeof(float) * kMlpParams));
    TRY(dL.alloc(sizeof(float) * epochs));
    TRY(cudaMemcpy(dW.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(dS.p, samples, sizeof(float) * AST_RECORD_FLOATS * n, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(dI.p, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    TRY(cudaMemset(dG.p, 0, sizeof(float) * kMlpParams));
    TRY(cudaMemset(dM1.p, 0, sizeof(float) * kMlpParams));
    TRY(cudaMemset(dM2.p, 0, sizeof(float) * kMlpParams));
    TRY(cudaMemset(dL.p, 0, sizeof(float) * epochs));
    std::vector<int64_t> order(nb);
    const float b1 = 0.9f, b2 = 0.999f;
    long long t = 0;
    for (int e = 0; e < epochs; e++) {
        for (int64_t i = 0; i < nb; i++) order[i] = i;
        std::shuffle(order.begin(), order.end(), gen);
        for (int64_t bi = 0; bi < nb; bi++) {
            mlp_grad_kernel<<<batch / kB, kB, sizeof(GradSmem)>>>(dW.as<float>(), dS.as<float>(), dI.as<int>(),
                                                                  order[bi] * batch, batch, 1.0f / (float)batch,
                                                                  dG.as<float>(), dL.as<float>() + e);
            t++;
            const float c1 = 1.0f / (1.0f - std::pow(b1, (float)t));
            const float c2 = 1.0f / (1.0f - std::pow(b2, (float)t));
            adam_kernel<<<(kMlpParams + 255) / 256, 256>>>(dW.as<float>(), dG.as<float>(), dM1.as<float>(),
                                                          dM2.as<float>(), lr, b1, b2, 1e-8f, c1, c2);
        }
        TRY(cudaGetLastError());
    }
    TRY(cudaMemcpy(params, dW.p, sizeof(float) * kMlpParams, cudaMemcpyDeviceToHost));
    if (loss_per_epoch) {
        TRY(cudaMemcpy(loss_per_epoch, dL.p, sizeof(float) * epochs, cudaMemcpyDeviceToHost));
        for (int e = 0; e < epochs; e++) loss_per_epoch[e] /= (float)(nb * batch);
    }
    return AST_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ tensor-core inference on given inputs
namespace {

// the step kernel's inference path (tc::forward16, 16 faces per warp tile)
// applied to n given feature rows; one warp per tile
__global__ void mlp_forward_tc_kernel(const float* __restrict__ W_g, const float* __restrict__ x, long long n,
                                      int stride, float* __restrict__ y)
{
    __shared__ float V[kVLen];
    __shared__ unsigned B1[tc::kL1], B2[tc::kL2];
    __shared__ float X[4][16][8];
    __shared__ float Y[4][16];
    for (int i = threadIdx.x; i < kVLen; i += blockDim.x) V[i] = mlp_vec(W_g, i);
    tc::pack_weights(W_g, B1, B2);
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const long long t0 = ((long long)blockIdx.x * 4 + w) * 16;
    if (lane < 16) {
        const long long k = t0 + lane;
        for (int i = 0; i < kMlpIn; i++) {
            const float v = (k < n) ? mlp_map(i, x[k * stride + i]) : 0.0f;
            X[w][lane][i] = fminf(fmaxf((v - V[kVShift + i]) * V[kVScale + i], -30.0f), 30.0f);
        }
        X[w][lane][6] = 0.0f;
        X[w][lane][7] = 0.0f;
    }
    __syncwarp();
    tc::forward16(V, B1, B2, X[w], Y[w]);
    __syncwarp();
    if (lane < 16 && t0 + lane < n) y[t0 + lane] = Y[w][lane];
}

}  // namespace

namespace {
// the packed network after the parameter block of a device copy
__global__ void __launch_bounds__(256) mlp_pack_kernel(float* W) { pack_network(W); }
}  // namespace

namespace ast {
int launch_mlp_pack(float* W, cudaStream_t st)
{
    mlp_pack_kernel<<<1, 256, 0, st>>>(W);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "network packing kernel launch");
}
}  // namespace ast

extern "C" int ast_mlp_forward_tc(const float* params, const float* x, int64_t n, int stride, float* y)
{
    if (!params || !x || !y || n < 1 || stride < kI) return AST_ERR_INVALID;
    DevBuf dW, dX, dY;
    TRY(dW.alloc(sizeof(float) * kMlpParams));
    TRY(dX.alloc(sizeof(float) * stride * n));
    TRY(dY.alloc(sizeof(float) * n));
    TRY(cudaMemcpy(dW.p, params, sizeof(float) * kMlpParams, cudaMemcpyHostToDevice));
    TRY(cudaMemcpy(dX.p, x, sizeof(float) * stride * n, cudaMemcpyHostToDevice));
    mlp_forward_tc_kernel<<<(int)((n + 63) / 64), 128>>>(dW.as<float>(), dX.as<float>(), n, stride, dY.as<float>());
    TRY(cudaGetLastError());
    TRY(cudaMemcpy(y, dY.p, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return AST_OK;
}
