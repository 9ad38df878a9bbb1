// convert.cuh - conversion between the reference's AoS double2 layout
// (s[k] = (rho, p), u[k] = (v_z, v_r), k = m*N + n) and the internal SoA
// planes (rho, p, v_z, v_r; rows of ld elements, planes of `plane`).
#pragma once

#include <cuda_runtime.h>

namespace ast {
// internal linkage: every translation unit that converts has its own copy

// cells k0 <= k < k1 (k1 = 0: the whole grid)
template <typename R>
static __global__ void aos_to_soa(const double2* __restrict__ s, const double2* __restrict__ u, R* __restrict__ q,
                           int N, int M, long long ld, long long plane, long long k0 = 0, long long k1 = 0)
{
    long long k = k0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (k1 > 0 ? k1 : (long long)N * M)) return;
    int m = (int)(k / N), n = (int)(k - (long long)m * N);
    long long o = (long long)m * ld + n;
    double2 a = s[k], b = u[k];
    q[o] = (R)a.x; q[o + plane] = (R)a.y; q[o + 2 * plane] = (R)b.x; q[o + 3 * plane] = (R)b.y;
}

template <typename R>
static __global__ void soa_to_aos(const R* __restrict__ q, double2* __restrict__ s, double2* __restrict__ u, int N,
                           int M, long long ld, long long plane, long long k0 = 0, long long k1 = 0)
{
    long long k = k0 + (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (k1 > 0 ? k1 : (long long)N * M)) return;
    int m = (int)(k / N), n = (int)(k - (long long)m * N);
    long long o = (long long)m * ld + n;
    s[k] = make_double2((double)q[o], (double)q[o + plane]);
    u[k] = make_double2((double)q[o + 2 * plane], (double)q[o + 3 * plane]);
}

// The reference's nn2 (K double3, k = m*N + n; x and y read) as two SoA
// planes of the solver's precision and row pitch
template <typename R>
static __global__ void nn2_to_planes(const double* __restrict__ nn2, R* __restrict__ q, int N, int M, long long ld,
                                     long long plane)
{
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (long long)N * M) return;
    const int m = (int)(k / N), n = (int)(k - (long long)m * N);
    const long long j = (long long)m * ld + n;
    q[j] = (R)nn2[3 * k];
    q[j + plane] = (R)nn2[3 * k + 1];
}

}  // namespace ast
