// sweep.cuh - the FP32 solver's strip kernel: each warp steps a strip of
// cells by sweeping up its rows with the stencil in registers.
//
// A strip is 30 columns wide and kSH rows high.  Lane l holds column
// n0 - 1 + l (lanes 0 and 31 hold the columns either side of the strip) and
// walks up the rows m0 .. m1 - 1.  At row m a lane keeps the cells of rows
// m, m+1, m+2 of its column in registers (the next row is loaded one step
// ahead), and per step it
//   - reconstructs its cell of row m+1 along r (minmod, once per cell): the
//     bottom value meets the top value of row m, kept from the step before,
//     at the r face m+1/2;
//   - reconstructs its cell of row m along z (once per cell), with the
//     neighbouring columns' cells from the neighbouring lanes (shuffles; the
//     outer neighbours of lanes 0 and 31 are loaded): its right value and
//     the right neighbour's left value meet at the z face right of the cell;
//   - evaluates those two faces (HLL: both at once in packed FP32) and
//     updates its cell of row m from the z faces left (the left lane's) and
//     right and the r faces below (kept from the step before) and above.
// Every face is evaluated once (the z faces of lanes 0 and 30 are also
// evaluated by the neighbouring strips), every cell is reconstructed once
// per direction, and the fluxes never leave registers: no shared memory and
// no barriers in the sweep.  Lanes 0 and 31 update nothing.
//
// The arithmetic of every face and cell is that of the tile kernels (the
// same reconstruction, flux functions, positivity rule, update and FP64
// islands in the same order), so the results are theirs bit for bit.
#pragma once

#include "mlp.cuh"
#include "step.cuh"

namespace ast {

constexpr int kSW = 30;   // columns a strip updates
constexpr int kSH = 32;   // rows of a strip (a multiple of the 16-row band unit)
constexpr unsigned kFull = 0xffffffffu;

// the four planes of a column: base pointers of its cell in row 0; cell
// (n, m) of the plane is base[k][m * ld] (32-bit row offsets: the planes
// of a grid that ast_config_check accepts hold fewer than 2^32 elements)
struct SwCol {
    const float* q[4];
    __device__ __forceinline__ void init(const StepParams& P, int n)
    {
        const float* b = (const float*)P.in + n;
        q[0] = b;
        q[1] = b + P.plane;
        q[2] = b + 2 * P.plane;
        q[3] = b + 3 * P.plane;
    }
};

// cell (n, m) of the FP32 input planes; strips at the grid's edge take the
// ghost rules (fetch_cell), the others plain loads through the column's
// plane bases (col: column n)
__device__ __forceinline__ void sw_load(const StepParams& P, bool edge, const SwCol& col, int n, int m, float v[4],
                                        int dn = 0)
{
    if (edge) {
        fetch_cell<float, kSoA>(P, n + dn, m, v);
        return;
    }
    const long long o = (long long)((unsigned)m * (unsigned)P.ld) + dn;
    v[0] = __ldg(col.q[0] + o);
    v[1] = __ldg(col.q[1] + o);
    v[2] = __ldg(col.q[2] + o);
    v[3] = __ldg(col.q[3] + o);
}

// the two face values of a cell t from its neighbours a (lower) and b
// (upper) along one direction: minmod reconstruction with the positivity
// rule of the tile kernels (a reconstructed rho or p <= 0, or p with grad_p
// off, takes the cell value)
template <bool RECON>
__device__ __forceinline__ void sw_recon(const StepParams& P, const float a[4], const float t[4], const float b[4],
                                         float lo[4], float hi[4])
{
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (RECON) {
            recon_pair(a[k], t[k], b[k], lo[k], hi[k]);
        } else {
            lo[k] = t[k];
            hi[k] = t[k];
        }
    }
    if (RECON) {
        if (lo[0] <= 0.0f) lo[0] = t[0];
        if (hi[0] <= 0.0f) hi[0] = t[0];
        if (lo[1] <= 0.0f || !P.grad_p) lo[1] = t[1];
        if (hi[1] <= 0.0f || !P.grad_p) hi[1] = t[1];
    }
}

// cell (n, m) can be updated: inside the grid and not held fixed
__device__ __forceinline__ bool sw_fixed(const StepParams& P, bool near, int n, int m)
{
    return near && n >= 0 && n < P.N && m >= 0 && m < P.M && cell_fixed(P, P.x_min + n * P.dx, P.y_min + m * P.dy);
}

// flux of one face of the HLLC family from its two sides in the face frame
// (rho, p, normal, tangential velocity), as face_flux evaluates it: the
// high-order flux in the region, HLL outside it
template <int FLUX>
__device__ __forceinline__ float sw_flux1(const Gas<float>& g, bool hi, const float L[4], const float U[4], float F[4])
{
    if (FLUX == 1 && hi) return flux_hllc(g, L[0], L[1], L[2], L[3], U[0], U[1], U[2], U[3], F);
    if (FLUX == 3 && hi) return flux_hllc_a(g, L[0], L[1], L[2], L[3], U[0], U[1], U[2], U[3], F);
    return flux_hll(g, L[0], L[1], L[2], L[3], U[0], U[1], U[2], U[3], F);
}

// out = (hi ? a : b) element by element, in registers
__device__ __forceinline__ void sw_sel(bool hi, const float a[4], const float b[4], float out[4])
{
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = hi ? a[k] : b[k];
}

// The start-value network in shared memory for the strip kernel, laid out
// for a warp that evaluates one face at a time with lane j computing hidden
// unit j of both layers: W1 and W2 transposed, so that the 32 lanes read 32
// consecutive words
struct SweepNet {
    float shift[kMlpIn], scale[kMlpIn];
    float w1t[kMlpIn][kMlpH];   // [input][unit]
    float b1[kMlpH];
    float w2t[kMlpH][kMlpH];    // [unit of layer 1][unit of layer 2]
    float b2[kMlpH], w3[kMlpH];
    float b3;
};

// the CTA's copy of the parameter block W (all threads; a barrier follows)
__device__ __forceinline__ void sweep_stage_net(const float* __restrict__ W, SweepNet& n)
{
    for (int i = threadIdx.x; i < kMlpH * kMlpH; i += blockDim.x) {
        const int k = i / kMlpH, j = i - k * kMlpH;
        n.w2t[k][j] = W[kOffW2 + j * kMlpH + k];
    }
    for (int i = threadIdx.x; i < kMlpIn * kMlpH; i += blockDim.x) {
        const int in = i / kMlpH, j = i - in * kMlpH;
        n.w1t[in][j] = W[kOffW1 + j * kMlpIn + in];
    }
    for (int j = threadIdx.x; j < kMlpH; j += blockDim.x) {
        n.b1[j] = W[kOffB1 + j];
        n.b2[j] = W[kOffB2 + j];
        n.w3[j] = W[kOffW3 + j];
    }
    if (threadIdx.x < kMlpIn) {
        n.shift[threadIdx.x] = W[kOffShift + threadIdx.x];
        n.scale[threadIdx.x] = W[kOffScale + threadIdx.x];
    }
    if (threadIdx.x == 0) n.b3 = W[kOffB3];
}

// y = log(p*/p_L) of the face whose features x lane `src` holds, evaluated
// by the whole warp in FP32 (the network of mlp_forward, the input map and
// standardisation included; the standardised inputs clamped to +-30 as the
// tile kernels' inference clamps them); every lane returns y
__device__ __forceinline__ float sweep_net(const SweepNet& n, const float x[kMlpIn], int src)
{
    const int j = threadIdx.x & 31;
    float z = n.b1[j];
#pragma unroll
    for (int i = 0; i < kMlpIn; i++) {
        const float xi = __shfl_sync(kFull, x[i], src);
        const float v = fminf(fmaxf((mlp_map(i, xi) - n.shift[i]) * n.scale[i], -30.0f), 30.0f);
        z = fmaf(n.w1t[i][j], v, z);
    }
    const float h1 = silu(z);
    float z2 = n.b2[j];
#pragma unroll 8
    for (int k = 0; k < kMlpH; k++) z2 = fmaf(n.w2t[k][j], __shfl_sync(kFull, h1, k), z2);
    float y = n.w3[j] * silu(z2);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) y += __shfl_xor_sync(kFull, y, o);
    return y + n.b3;
}

// The exact-solver flux of one face from its sides a (lower) and b (upper)
// in the face frame, as the tile kernels evaluate it (face_flux, then for
// the iterative patterns queue_pass): HLL outside the high-order region;
// identical sides in closed form; patterns 0 and 1 sampled directly;
// patterns 2 and 3 by the safeguarded Newton from the acoustic start value
// or, for faces above the gate in the learned form, from the network's
// (evaluated by the whole warp, one face at a time).  Called by the whole
// warp (the network needs every lane).
__device__ __forceinline__ float sw_godunov_face(const StepParams& P, const Gas<float>& g, bool hi, bool learned,
                                                 const SweepNet* net, const float a[4], const float b[4], float F[4],
                                                 RiemannCount& rc, int& fallback)
{
    const bool ident = hi && a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3];
    RPre<float> q;
    q.pattern = 4;
    if (hi && !ident) q = godunov_pre(g, a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3]);
    const bool iter = hi && !ident && (q.pattern == 2 || q.pattern == 3);
    const bool strong = iter && wave_strength(q) > P.mlp_gate;
    float p0m = 0.0f;
    if (learned) {
        unsigned mask = __ballot_sync(kFull, strong);
        if (mask) {
            float x[kMlpIn] = {1.0f, 1.0f, 0.0f, 1.0f, 1.0f, 0.0f};
            float pL = 1.0f;
            if (strong) {
                float rL, uL, cL, rR, pR, uR, cR;
                face_sides(q, rL, pL, uL, cL, rR, pR, uR, cR);
                mlp_features(g.ga, rL, pL, uL, cL, rR, pR, uR, cR, x);
            }
            while (mask) {
                const int src = __ffs(mask) - 1;
                const float y = sweep_net(*net, x, src);
                if ((int)(threadIdx.x & 31) == src) p0m = pL * __expf(y);
                mask &= mask - 1u;
            }
        }
    }
    if (!hi) return flux_hll(g, a[0], a[1], a[2], a[3], b[0], b[1], b[2], b[3], F);
    if (ident) {
        // identical states: the exact solution is that state, its flux the
        // physical flux, its largest wave speed |u_n| + c
        const float r = a[0], p = a[1], un = a[2], ut = a[3];
        const float cs = sqrt(g.ga * p / r);
        const float m = r * un;
        F[0] = m;
        F[1] = m * un + p;
        F[2] = m * ut;
        F[3] = un * (p * g.inv_g1 + 0.5f * r * (un * un + ut * ut) + p);
        return fmaxf(fabsf(un) + cs, g.eps8);
    }
    if (iter) {
        const float p = solve_queued(P, g, q, strong, p0m, rc, fallback);
        return godunov_sample<float, kSampleIterative>(g, q, p, F, rc);
    }
    return godunov_sample<float, kSampleClosed>(g, q, 0.0f, F, rc);
}

// One strip: columns n0 .. n0+29 (lanes 1..30), rows [m0, m1).  Called by
// a whole warp.
template <int FLUX, bool RECON>
__device__ __forceinline__ void sweep_strip(const StepParams& P, const StepConsts& K, int n0, int m0, int m1,
                                            const SweepNet* net, TileAcc<float>& acc)
{
    const Gas<float>& g = P.gf;
    const bool learned = FLUX == 2 && P.guess == 1 && P.mlp != nullptr;
    const int lane = threadIdx.x & 31;
    const int c = n0 - 1 + lane;
    const int N = P.N, M = P.M;
    // every load of the strip (columns n0-2 .. n0+31, rows m0-2 .. m1+2)
    // inside the grid, or the ghost rules on every load
    const bool edge = n0 - 2 < 0 || n0 + kSW + 1 >= N || m0 - 2 < 0 || m1 + 2 >= M;
    const bool near = P.fixed_region && n0 - 2 <= P.fixed_nhi && n0 + kSW + 1 >= P.fixed_nlo && m0 - 2 <= P.fixed_mhi;
    const bool cin = c >= 0 && c < N;
    const bool owner = lane >= 1 && lane <= kSW && c < N;
    // the outer z neighbour of lanes 0 and 31, column c + dx (the other
    // lanes load their own cell again, an L1 hit, and do not use it)
    const int dx = (lane == 0) ? -1 : (lane == 31 ? 1 : 0);
    SwCol cc;
    if (!edge) cc.init(P, c);
    // region test of this lane's faces (lower cell's column, as face_meta)
    const bool hz = !P.region_select || (c >= P.region_zlo && c <= P.region_zhi);
    const bool hr = !P.region_select || (c >= P.region_rlo && c <= P.region_rhi);

    float w0[4], w1[4], w2[4], ex[4];
    float Rr[4], Fb[4];
    bool fx0, fx1;
    {
        // warm-up: rows m0-2 .. m0+2, the r face below row m0
        float a[4], b[4];
        sw_load(P, edge, cc, c, m0 - 2, a);
        sw_load(P, edge, cc, c, m0 - 1, b);
        sw_load(P, edge, cc, c, m0, w0);
        sw_load(P, edge, cc, c, m0 + 1, w1);
        sw_load(P, edge, cc, c, m0 + 2, w2);
        sw_load(P, edge, cc, c, m0, ex, dx);
        float lo[4], Rm[4];
        sw_recon<RECON>(P, a, b, w0, lo, Rm);   // cell m0-1: its top value
        sw_recon<RECON>(P, b, w0, w1, lo, Rr);  // cell m0: bottom (lo), top (Rr)
        // r face m0 - 1/2 between rows m0-1 (b) and m0 (w0), face frame
        float L[4], U[4];
        sw_sel(hr, Rm, b, L);
        sw_sel(hr, lo, w0, U);
        float F[4];
        float Sp;
        if (FLUX == 0) {
            // the packed HLL of the other faces (each element rounds as they do)
            float2 F2[4], S2;
            flux_hll_x2(g, pk(L[0], L[0]), pk(L[1], L[1]), pk(L[3], L[3]), pk(L[2], L[2]), pk(U[0], U[0]),
                        pk(U[1], U[1]), pk(U[3], U[3]), pk(U[2], U[2]), F2, S2);
            F[0] = F2[0].x; F[1] = F2[1].x; F[2] = F2[2].x; F[3] = F2[3].x;
            Sp = S2.x;
        } else {
            const float Lf[4] = {L[0], L[1], L[3], L[2]}, Uf[4] = {U[0], U[1], U[3], U[2]};
            if constexpr (FLUX == 2)
                Sp = sw_godunov_face(P, g, hr, learned, net, Lf, Uf, F, acc.rc, acc.fallback);
            else
                Sp = sw_flux1<FLUX>(g, hr, Lf, Uf, F);
        }
        Fb[0] = F[0]; Fb[1] = F[2]; Fb[2] = F[1]; Fb[3] = F[3];
        const bool fxb = sw_fixed(P, near, c, m0 - 1);
        fx0 = sw_fixed(P, near, c, m0);
        const bool act = cin && ((m0 - 1 >= 0 && !fxb) || !fx0);
        if (act) {
            if (!(Sp == Sp)) { acc.rc.status |= 0x10u; Sp = 0.0f; }
            acc.smr = fmaxf(acc.smr, Sp);
        }
    }
    const float gaf = g.ga, g1f = g.g1, ig1f = g.inv_g1;
#pragma unroll 1
    for (int m = m0; m < m1; m++) {
        // row m+3 and the outer neighbour of row m+1, one step ahead
        float nx[4], exn[4];
        sw_load(P, edge, cc, c, m + 3, nx);
        sw_load(P, edge, cc, c, m + 1, exn, dx);
        fx1 = sw_fixed(P, near, c, m + 1);
        // r: cell m+1 (rows m, m+1, m+2)
        float Lr1[4], Rr1[4];
        sw_recon<RECON>(P, w0, w1, w2, Lr1, Rr1);
        // z: cell m with its left and right neighbours
        float zl[4], zr[4], Lz[4], Rz[4], Un[4], Uc[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            zl[k] = __shfl_up_sync(kFull, w0[k], 1);
            zr[k] = __shfl_down_sync(kFull, w0[k], 1);
            if (lane == 0) zl[k] = ex[k];
            if (lane == 31) zr[k] = ex[k];
        }
        sw_recon<RECON>(P, zl, w0, zr, Lz, Rz);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            Un[k] = __shfl_down_sync(kFull, Lz[k], 1);   // right neighbour's left value
            Uc[k] = zr[k];                               // right neighbour's cell value
        }
        // the two faces: z face right of cell m (zL | zU) and r face above it
        float zL[4], zU[4], rL[4], rU[4];
        if (P.region_select) {
            sw_sel(hz, Rz, w0, zL);
            sw_sel(hz, Un, Uc, zU);
            sw_sel(hr, Rr, w0, rL);
            sw_sel(hr, Lr1, w1, rU);
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                zL[k] = Rz[k];
                zU[k] = Un[k];
                rL[k] = Rr[k];
                rU[k] = Lr1[k];
            }
        }
        float Fz[4], Ft[4], Sz, Sr;
        if constexpr (FLUX == 0) {
            float2 F[4], S;
            flux_hll_x2(g, pk(zL[0], rL[0]), pk(zL[1], rL[1]), pk(zL[2], rL[3]), pk(zL[3], rL[2]), pk(zU[0], rU[0]),
                        pk(zU[1], rU[1]), pk(zU[2], rU[3]), pk(zU[3], rU[2]), F, S);
            Fz[0] = F[0].x; Fz[1] = F[1].x; Fz[2] = F[2].x; Fz[3] = F[3].x;
            Ft[0] = F[0].y; Ft[1] = F[2].y; Ft[2] = F[1].y; Ft[3] = F[3].y;
            Sz = S.x;
            Sr = S.y;
        } else {
            // one flux call site for both faces (a smaller kernel)
            // (face frames: z (rho, p, v_z, v_r), r (rho, p, v_r, v_z))
            const float zLf[4] = {zL[0], zL[1], zL[2], zL[3]}, zUf[4] = {zU[0], zU[1], zU[2], zU[3]};
            const float rLf[4] = {rL[0], rL[1], rL[3], rL[2]}, rUf[4] = {rU[0], rU[1], rU[3], rU[2]};
            float Fo0[4], Fo1[4], So0 = 0.0f, So1 = 0.0f;
#pragma unroll 1
            for (int s = 0; s < 2; s++) {
                float a[4], b[4], F[4];
                sw_sel(s != 0, rLf, zLf, a);
                sw_sel(s != 0, rUf, zUf, b);
                float Sp;
                if constexpr (FLUX == 2)
                    Sp = sw_godunov_face(P, g, s ? hr : hz, learned, net, a, b, F, acc.rc, acc.fallback);
                else
                    Sp = sw_flux1<FLUX>(g, s ? hr : hz, a, b, F);
                if (s) {
                    Fo1[0] = F[0]; Fo1[1] = F[1]; Fo1[2] = F[2]; Fo1[3] = F[3]; So1 = Sp;
                } else {
                    Fo0[0] = F[0]; Fo0[1] = F[1]; Fo0[2] = F[2]; Fo0[3] = F[3]; So0 = Sp;
                }
            }
            Fz[0] = Fo0[0]; Fz[1] = Fo0[1]; Fz[2] = Fo0[2]; Fz[3] = Fo0[3];
            Ft[0] = Fo1[0]; Ft[1] = Fo1[2]; Ft[2] = Fo1[1]; Ft[3] = Fo1[3];
            Sz = So0;
            Sr = So1;
        }
        // wave speeds of the faces that belong to an updated cell
        const bool fxr = __shfl_down_sync(kFull, fx0 ? 1 : 0, 1) != 0;
        const bool actz = lane <= kSW && ((cin && !fx0) || (c + 1 >= 0 && c + 1 < N && !fxr));
        const bool actr = cin && (!fx0 || (m + 1 < M && !fx1));
        if (actz) {
            if (!(Sz == Sz)) { acc.rc.status |= 0x10u; Sz = 0.0f; }
            acc.smz = fmaxf(acc.smz, Sz);
        }
        if (actr) {
            if (!(Sr == Sr)) { acc.rc.status |= 0x10u; Sr = 0.0f; }
            acc.smr = fmaxf(acc.smr, Sr);
        }
        // the z face left of the cell: the left lane's
        float Fl[4];
#pragma unroll
        for (int k = 0; k < 4; k++) Fl[k] = __shfl_up_sync(kFull, Fz[k], 1);
        // the update of cell (c, m)
        if (owner) {
            float o[4] = {w0[0], w0[1], w0[2], w0[3]};
            if (!fx0) {
                const float f[4][4] = {{Fz[0], Fl[0], Fb[0], Ft[0]},
                                       {Fz[1], Fl[1], Fb[1], Ft[1]},
                                       {Fz[2], Fl[2], Fb[2], Ft[2]},
                                       {Fz[3], Fl[3], Fb[3], Ft[3]}};
                if (P.geom == 1 && m < 4) {
                    // the FP64 update of the four rows next to the axis
                    const double T_do = K.T_do;
                    const double y = P.y_min + m * P.dy;
                    double Q2 = 0.0;
                    if (P.body_force) {
                        const double x = P.x_min + c * P.dx;
                        if (x > P.body_lo && x < P.body_hi)
                            Q2 = (y >= P.body_rsplit) ? -P.body_amp * (double)w0[0] : P.body_amp * (double)w0[0];
                    }
                    update_cell<double>(P, P.gd.ga, P.gd.g1, P.gd.inv_g1, w0, f, T_do, K.tdv, T_do / y, P.dx, P.dy,
                                        Q2, 0.0, 0.0, acc.nrho, acc.np, acc.rc.status, o);
                } else {
                    const float y = P.y_minf + (float)m * P.dyf;
                    float Q2 = 0.0f;
                    if (P.body_force) {
                        const float x = P.x_minf + (float)c * P.dxf;
                        if (x > P.body_lof && x < P.body_hif)
                            Q2 = (y >= P.body_rsplitf) ? -P.body_ampf * w0[0] : P.body_ampf * w0[0];
                    }
                    const float ty = (P.geom == 1) ? K.T_f / y : 0.0f;
                    float E2, KE2;
                    update_cell<float>(P, gaf, g1f, ig1f, w0, f, K.T_f, K.tdv_f, ty, P.dxf, P.dyf, Q2, 0.0f, 0.0f,
                                       acc.nrho, acc.np, acc.rc.status, o, &E2, &KE2);
                    // pressure recovery in FP64 where the kinetic energy is
                    // more than 99% of the total
                    if (KE2 > 0.99f * E2)
                        o[1] = (float)pressure_fp64(P, w0, f, K.tdv_f, ty, K.T_f, Q2, P.dxf, P.dyf, acc.np);
                }
            }
            float* out = (float*)P.out + (long long)m * P.ld + c;
            out[0] = o[0];
            out[P.plane] = o[1];
            out[2 * P.plane] = o[2];
            out[3 * P.plane] = o[3];
        }
        // the window moves up one row
#pragma unroll
        for (int k = 0; k < 4; k++) {
            Rr[k] = Rr1[k];
            Fb[k] = Ft[k];
            w0[k] = w1[k];
            w1[k] = w2[k];
            w2[k] = nx[k];
            ex[k] = exn[k];
        }
        fx0 = fx1;
    }
}

// The FP32 solver's strip kernel: as many CTAs of 8 warps as fit, each warp
// taking strips from the counter in the clock (strips of a band of rows
// when P.band_hi > 0) until none are left.  The CTA's wave-speed maxima and
// counters are reported once (one ticket per CTA); the last CTA shifts the
// clock and rewinds the counter.
template <int FLUX, bool RECON>
__global__ void __launch_bounds__(kThreads, 2) sweep_kernel(StepParams P)
{
    __shared__ StepConsts sK;
    const SweepNet* net = nullptr;
    if constexpr (FLUX == 2) {
        // the learned form's network, staged once per CTA
        __shared__ SweepNet snet;
        if (P.guess == 1 && P.mlp != nullptr) sweep_stage_net(P.mlp, snet);
        net = &snet;
    }
    if (threadIdx.x == 0) step_consts(P, sK);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int r_lo = P.band_lo * 16;
    const int r_hi = P.band_hi > 0 ? min(P.band_hi * 16, P.M) : P.M;
    const int sz = (P.N + kSW - 1) / kSW;
    const int strips = sz * ((r_hi - r_lo + kSH - 1) / kSH);
    TileAcc<float> acc;
    acc.clear();
    for (;;) {
        int s = 0;
        if (lane == 0) s = (int)atomicAdd(&P.clock->next_tile, 1u);
        s = __shfl_sync(kFull, s, 0);
        if (s >= strips) break;
        const int n0 = (s % sz) * kSW;
        const int m0 = r_lo + (s / sz) * kSH;
        sweep_strip<FLUX, RECON>(P, sK, n0, m0, min(m0 + kSH, r_hi), net, acc);
    }
    cta_epilogue<float>(P, acc, P.units > 0 ? (unsigned)P.units : gridDim.x, true);
}

}  // namespace ast
