// scalar.cu - the passive scalar Q of the FP64 solver (ast_set_scalar).
//
// Q is a density carried by the flow (a tracer's mass per volume): the
// reference's HLLC solvers compute its face flux beside the gas flux (the Q
// channel of HLLC_2d_Korolkov_b_s, Gas_Dinamic.cu:1660-1808, and
// HLLCQ_Korolkov_2D, Gas_Dinamic.cu:249-353), but its step kernels never
// carry it (HLLC_2d_Korolkov passes Q = 1 and drops PQ, Gas_Dinamic.cu:1814-
// 1826).  Here it is carried: each step, before the gas step (which it does
// not change), scalar_kernel updates Q from the same old state with the
// same reconstruction, the same solver and the same update form as the
// density:
//
//   Q' = Q - T_do/(dx dy) * sum of face fluxes  [- T_do/r * Q * v_r]
//
// (the bracket on the axisymmetric grid, as the density's cylindrical
// source).  One thread per cell evaluates its four faces, each in the face
// frame with the lower cell on the left, so the two cells of a face compute
// the same bits and Q is conserved to rounding.  Ghost values of Q follow
// the state's rules: mirrored at REFLECT sides, copied from the boundary
// cell at OUTFLOW / SUCTION / NONREFLECT sides, cfg.scalar_in at FIXED
// sides.  Face values are reconstructed with the density's rule (minmod;
// a value <= 0 falls back to the cell's).  Cells held fixed keep Q.
#include <cuda_runtime.h>

#include "../../include/asteriy_gb300.h"
#include "launch.cuh"

using namespace ast;

namespace {

constexpr int kScalarThreads = 128;

// Q at (n, m), with the ghost rules of the side that (n, m) lies beyond
// (fetch_cell's index rules)
__device__ __forceinline__ double scalar_at(const StepParams& P, const double* __restrict__ q, double q_fixed, int n,
                                            int m)
{
    const int N = P.N, M = P.M;
    if (n >= 0 && n < N && m >= 0 && m < M) return q[(long long)m * N + n];
    int side, j, bn, bm, mn, mm;
    if (n < 0)       { side = 0; j = -1 - n; bn = 0;     bm = m; mn = j;         mm = m; }
    else if (n >= N) { side = 1; j = n - N;  bn = N - 1; bm = m; mn = N - 1 - j; mm = m; }
    else if (m < 0)  { side = 2; j = -1 - m; bn = n; bm = 0;     mn = n; mm = j; }
    else             { side = 3; j = m - M;  bn = n; bm = M - 1; mn = n; mm = M - 1 - j; }
    mn = min(max(mn, 0), N - 1);
    mm = min(max(mm, 0), M - 1);
    bm = min(max(bm, 0), M - 1);
    bn = min(max(bn, 0), N - 1);
    const int kind = P.bc_kind[side];
    if (kind == 0) return q[(long long)mm * N + mn];   // REFLECT
    if (kind == 2) return q_fixed;                      // FIXED
    return q[(long long)bm * N + bn];                   // OUTFLOW, SUCTION, NONREFLECT
}

// the scalar flux of the face between cells a (lower) and b (upper), with a's
// lower neighbour a0 and b's upper neighbour b1 (states as fetch_cell gives
// them, scalars beside); ZF: a z face (normal v_z)
template <int FLUX, bool RECON, bool ZF>
__device__ __forceinline__ double face_q(const StepParams& P, const Gas<double>& g, const double a0[4],
                                         const double a[4], const double b[4], const double b1[4], double qa0,
                                         double qa, double qb, double qb1)
{
    constexpr int NN = ZF ? 2 : 3, TT = ZF ? 3 : 2;
    double L[4], U[4];
    double QL = qa, QU = qb;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        L[k] = a[k];
        U[k] = b[k];
    }
    if (RECON) {
        // the step's face values (face_states / face_two): minmod, with the
        // positivity rule for rho and p (kernel.cu:2706-2743)
#pragma unroll
        for (int k = 0; k < 4; k++) {
            double x0, x1;
            recon_pair(a0[k], a[k], b[k], x0, x1);
            L[k] = x1;
            recon_pair(a[k], b[k], b1[k], x0, x1);
            U[k] = x0;
        }
        if (L[0] <= 0.0) L[0] = a[0];
        if (U[0] <= 0.0) U[0] = b[0];
        if (L[1] <= 0.0 || !P.grad_p) L[1] = a[1];
        if (U[1] <= 0.0 || !P.grad_p) U[1] = b[1];
        double x0, x1;
        recon_pair(qa0, qa, qb, x0, x1);
        QL = (x1 <= 0.0) ? qa : x1;
        recon_pair(qa, qb, qb1, x0, x1);
        QU = (x0 <= 0.0) ? qb : x0;
    }
    if constexpr (FLUX == 4) {
        double F[4], FQ;
        flux_hllcq(g, L[0], L[1], L[NN], L[TT], QL, U[0], U[1], U[NN], U[TT], QU, F, FQ);
        return FQ;
    } else {
        return flux_hllc_q(g, L[0], L[1], L[NN], QL, U[0], U[1], U[NN], QU);
    }
}

template <int FLUX, bool RECON>
__global__ void __launch_bounds__(kScalarThreads) scalar_kernel(StepParams P, const double* __restrict__ q,
                                                               double* __restrict__ q2, double q_fixed)
{
    const long long idx = (long long)blockIdx.x * kScalarThreads + threadIdx.x;
    if (idx >= (long long)P.N * P.M) return;
    const int n = (int)(idx % P.N), m = (int)(idx / P.N);
    const double q1 = q[idx];
    if (P.fixed_region && cell_fixed(P, P.x_min + n * P.dx, P.y_min + m * P.dy)) {
        q2[idx] = q1;
        return;
    }
    const Gas<double>& g = P.gd;
    // the cross stencil of radius 2: z neighbours n-2 .. n+2, r neighbours
    double zc[5][4], rc[4][4], zq[5], rq[4];   // rc / rq: rows m-2, m-1, m+1, m+2
#pragma unroll
    for (int i = 0; i < 5; i++) {
        fetch_cell<double, kSoA>(P, n - 2 + i, m, zc[i]);
        zq[i] = scalar_at(P, q, q_fixed, n - 2 + i, m);
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int mm = m + (i < 2 ? i - 2 : i - 1);
        fetch_cell<double, kSoA>(P, n, mm, rc[i]);
        rq[i] = scalar_at(P, q, q_fixed, n, mm);
    }
    // face fluxes along +z / +r: right, left, bottom, top
    const double f_r = face_q<FLUX, RECON, true>(P, g, zc[1], zc[2], zc[3], zc[4], zq[1], zq[2], zq[3], zq[4]);
    const double f_l = face_q<FLUX, RECON, true>(P, g, zc[0], zc[1], zc[2], zc[3], zq[0], zq[1], zq[2], zq[3]);
    const double f_b = face_q<FLUX, RECON, false>(P, g, rc[0], rc[1], zc[2], rc[2], rq[0], rq[1], zq[2], rq[2]);
    const double f_t = face_q<FLUX, RECON, false>(P, g, rc[1], zc[2], rc[2], rc[3], rq[1], zq[2], rq[2], rq[3]);
    // the density's update form (update_cell)
    const double T_do = (P.clock != nullptr) ? *(volatile double*)&P.clock->T_do : *P.T_do_ptr;
    const double tdv = T_do / (P.dx * P.dy);
    const double f12 = f_r, f14 = -f_l, f13 = -f_b, f15 = f_t;
    double out;
    if (P.geom == 1) {
        const double y = P.y_min + m * P.dy;
        const double ty = T_do / y;
        const double ps = (f12 + f14) * P.dy + (f13 + f15) * P.dx;
        out = q1 - tdv * ps - ty * q1 * zc[2][3];
    } else {
        const double ps = f12 * P.dy + f13 * P.dx + f14 * P.dy + f15 * P.dx;
        out = q1 - tdv * ps;
    }
    q2[idx] = out;
}

}  // namespace

namespace ast {

int launch_scalar(const StepParams& P, const double* q, double* q2, int flux, int recon, double q_fixed,
                  cudaStream_t st)
{
    const long long K = (long long)P.N * P.M;
    const unsigned nb = (unsigned)((K + kScalarThreads - 1) / kScalarThreads);
    if (flux == AST_FLUX_HLLCQ) {
        if (recon) scalar_kernel<4, true><<<nb, kScalarThreads, 0, st>>>(P, q, q2, q_fixed);
        else scalar_kernel<4, false><<<nb, kScalarThreads, 0, st>>>(P, q, q2, q_fixed);
    } else if (flux == AST_FLUX_HLLC) {
        if (recon) scalar_kernel<1, true><<<nb, kScalarThreads, 0, st>>>(P, q, q2, q_fixed);
        else scalar_kernel<1, false><<<nb, kScalarThreads, 0, st>>>(P, q, q2, q_fixed);
    } else {
        return set_error(AST_ERR_UNSUPPORTED, "the passive scalar needs the HLLC or HLLCQ flux");
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "scalar kernel launch");
}

}  // namespace ast
