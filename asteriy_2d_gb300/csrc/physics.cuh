// physics.cuh - face fluxes and reconstruction for the r-z step, on the GPU.
//
// Every face is evaluated once, in its own frame: the normal points from
// the lower-index cell L to the higher-index cell R (+z for z faces, +r for
// r faces), un/ut are the normal/tangential velocities, and a flux is
// returned as (mass, normal momentum, tangential momentum, energy).  The
// reference evaluates each face twice, once from each cell with that cell's
// outward normal; HLL is exactly antisymmetric under that exchange, the
// other solvers to rounding.
//
// Algorithms follow the reference:
//   minmod ............ kernel.cu:22-33, sign Gas_Dinamic.cu:858-872
//   HLL ............... kernel.cu:1399-1523 (Davis bounds, Omega = 0)
//   HLLC .............. Gas_Dinamic.cu:1604-1811 (metod 2, W = 0, tangential
//                       velocity kept per side, nul_potok = false)
//   exact Godunov ..... kernel.cu:128-570 with newton :635-680,
//                       devtwo :682-749, lev :751-765
// Each solver returns the wave speed S whose dt candidate the reference
// forms as krit*rad/S; the step kernel reduces max S per direction and
// divides once (division by a positive S is monotone, so
// min(krit*rad/S_i) == krit*rad/max(S_i) exactly).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace ast {

template <typename R>
struct Gas {
    R ga, g1, g2, gp, gm;     // gamma, gamma-1, gamma+1, (g2/ga)/2, (g1/ga)/2
    R inv_g1;                 // 1/(gamma-1)
    R tol;                    // Newton / bisection tolerance
    R eps;                    // 10e-10: degenerate rarefaction test (Header.h:62)
    R eps8;                   // 10e-8: smallest wave speed for dt (Header.h:63)
    int max_iter;
};

template <typename R>
__host__ __device__ inline Gas<R> make_gas(double gamma, double tol, int max_iter)
{
    Gas<R> g;
    double g1 = gamma - 1.0, g2 = gamma + 1.0;
    g.ga = (R)gamma;
    g.g1 = (R)g1;
    g.g2 = (R)g2;
    g.gp = (R)((g2 / gamma) / 2.0);
    g.gm = (R)((g1 / gamma) / 2.0);
    g.inv_g1 = (R)(1.0 / g1);
    g.tol = (R)tol;
    g.eps = (R)10e-10;
    g.eps8 = (R)10e-8;
    g.max_iter = max_iter;
    return g;
}

// per-thread counters of Riemann-solver work (summed per warp by the caller)
struct RiemannCount {
    int newton_calls, newton_iters, bisect_calls, bisect_iters;
    int newton_max;
    int strong_calls, strong_iters;   // faces above the learned-start gate
    unsigned status;
    __device__ void clear()
    {
        newton_calls = newton_iters = bisect_calls = bisect_iters = newton_max = 0;
        strong_calls = strong_iters = 0;
        status = 0;
    }
};

// ------------------------------------------------------------------ minmod
// (sign a + sign b)/2 * min(|a|, |b|): zero unless both have one sign,
// as sign(a) max(0, min(|a|, sign(a) b)) (the same value; a zero result may
// differ in the sign of zero only), the products with sign(a) taken as
// sign-bit operations
__device__ __forceinline__ float minmod_d(float a, float b)
{
    const unsigned sa = __float_as_uint(a) & 0x80000000u;
    const float m = fmaxf(0.0f, fminf(fabsf(a), __uint_as_float(__float_as_uint(b) ^ sa)));
    return __uint_as_float(__float_as_uint(m) | sa);
}
__device__ __forceinline__ double minmod_d(double a, double b)
{
    const unsigned long long sa = (unsigned long long)__double_as_longlong(a) & 0x8000000000000000ull;
    const double bs = __longlong_as_double((long long)((unsigned long long)__double_as_longlong(b) ^ sa));
    const double m = fmax(0.0, fmin(fabs(a), bs));
    return __longlong_as_double((long long)((unsigned long long)__double_as_longlong(m) | sa));
}

// left / right face values of a cell from its three-point stencil; the
// reference's linear2 with the coordinate differences folded in
template <typename R>
__device__ __forceinline__ void recon_pair(R tm, R t0, R tp, R& left, R& right)
{
    R d = minmod_d(t0 - tm, tp - t0) * R(0.5);
    left = t0 - d;
    right = t0 + d;
}

// ------------------------------------------------------------------ HLL
template <typename R>
__device__ __forceinline__ R flux_hll(const Gas<R>& g, R rL, R pL, R unL, R utL, R rR, R pR, R unR, R utR,
                                      R F[4])
{
    R cL = (rL <= R(0)) ? R(0) : sqrt(g.ga * pL / rL);
    R cR = (rR <= R(0)) ? R(0) : sqrt(g.ga * pR / rR);
    R eL = pL * g.inv_g1 + rL * (unL * unL + utL * utL) * R(0.5);
    R eR = pR * g.inv_g1 + rR * (unR * unR + utR * utR) * R(0.5);
    // the reference's selects, not fmin/fmax: they give the same values,
    // and a NaN (the sound speed of a negative pressure) propagates or not
    // as in the reference (kernel.cu:1399-1523)
    R mxc = (cL >= cR) ? cL : cR;
    R DL = ((unL <= unR) ? unL : unR) - mxc;
    R DR = ((unL >= unR) ? unL : unR) + mxc;
    R S = (fabs(DL) >= fabs(DR)) ? fabs(DL) : fabs(DR);
    R mL = rL * unL, mR = rR * unR;
    if (DL > R(0)) {
        F[0] = mL; F[1] = mL * unL + pL; F[2] = mL * utL; F[3] = (eL + pL) * unL;
    } else if (DR < R(0)) {
        F[0] = mR; F[1] = mR * unR + pR; F[2] = mR * utR; F[3] = (eR + pR) * unR;
    } else {
        R fl0 = mL, fl1 = mL * unL + pL, fl2 = mL * utL, fl3 = (eL + pL) * unL;
        R fr0 = mR, fr1 = mR * unR + pR, fr2 = mR * utR, fr3 = (eR + pR) * unR;
        R inv = R(1) / (DR - DL);
        R dd = DL * DR;
        F[0] = (DR * fl0 - DL * fr0 + dd * (rR - rL)) * inv;
        F[1] = (DR * fl1 - DL * fr1 + dd * (mR - mL)) * inv;
        F[2] = (DR * fl2 - DL * fr2 + dd * (rR * utR - rL * utL)) * inv;
        F[3] = (DR * fl3 - DL * fr3 + dd * (eR - eL)) * inv;
    }
    return S;
}

// ------------------------------------------------------------------ identical states
// The HLL and HLLC fluxes of a face whose two sides hold one state (r, p,
// un, ut), r > 0, p > 0: the physical flux of that state, which their
// formulas reach up to rounding (and exactly on supersonic faces, with these
// expressions), and the wave speed they return, max(|un - c|, |un + c|)
// with c = sqrt(ga p / r), formed as they form it.
template <typename R>
__device__ __forceinline__ R flux_physical(const Gas<R>& g, R r, R p, R un, R ut, R F[4])
{
    const R c = sqrt(g.ga * p / r);
    const R SL = un - c, SR = un + c;
    const R e = p * g.inv_g1 + r * (un * un + ut * ut) * R(0.5);
    const R m = r * un;
    F[0] = m;
    F[1] = m * un + p;
    F[2] = m * ut;
    F[3] = (e + p) * un;
    return fmax(fabs(SL), fabs(SR));
}

// ------------------------------------------------------------------ HLL, two faces in packed FP32
// Two independent HLL faces (.x and .y) with each add, multiply and fused
// multiply-add on the pair issued as one packed FP32 instruction (FADD2,
// FMUL2, FFMA2); divisions, square roots, min/max and the selects stay per
// element.  The same formula as flux_hll, with the multiply-adds fused
// explicitly; each element rounds as a scalar evaluation with those fusions.
__device__ __forceinline__ float2 pk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }

__device__ __forceinline__ void flux_hll_x2(const Gas<float>& g, float2 rL, float2 pL, float2 unL, float2 utL,
                                            float2 rR, float2 pR, float2 unR, float2 utR, float2 F[4], float2& S)
{
    const float2 ga = pk(g.ga, g.ga), ig1 = pk(g.inv_g1, g.inv_g1), half = pk(0.5f, 0.5f);
    const float2 gpL = mul2(ga, pL), gpR = mul2(ga, pR);
    const float2 cL = pk((rL.x <= 0.0f) ? 0.0f : sqrtf(gpL.x / rL.x), (rL.y <= 0.0f) ? 0.0f : sqrtf(gpL.y / rL.y));
    const float2 cR = pk((rR.x <= 0.0f) ? 0.0f : sqrtf(gpR.x / rR.x), (rR.y <= 0.0f) ? 0.0f : sqrtf(gpR.y / rR.y));
    const float2 eL = fma2(mul2(rL, fma2(utL, utL, mul2(unL, unL))), half, mul2(pL, ig1));
    const float2 eR = fma2(mul2(rR, fma2(utR, utR, mul2(unR, unR))), half, mul2(pR, ig1));
    const float2 mxc = pk(fmaxf(cL.x, cR.x), fmaxf(cL.y, cR.y));
    const float2 DL = sub2(pk(fminf(unL.x, unR.x), fminf(unL.y, unR.y)), mxc);
    const float2 DR = add2(pk(fmaxf(unL.x, unR.x), fmaxf(unL.y, unR.y)), mxc);
    S = pk(fmaxf(fabsf(DL.x), fabsf(DR.x)), fmaxf(fabsf(DL.y), fabsf(DR.y)));
    const float2 mL = mul2(rL, unL), mR = mul2(rR, unR);
    const float2 fl1 = fma2(mL, unL, pL), fl2 = mul2(mL, utL), fl3 = mul2(add2(eL, pL), unL);
    const float2 fr1 = fma2(mR, unR, pR), fr2 = mul2(mR, utR), fr3 = mul2(add2(eR, pR), unR);
    const float2 d = sub2(DR, DL);
    const float2 inv = pk(1.0f / d.x, 1.0f / d.y);
    const float2 dd = mul2(DL, DR);
    const float2 nDL = mul2(DL, pk(-1.0f, -1.0f));
    F[0] = mul2(fma2(dd, sub2(rR, rL), fma2(nDL, mR, mul2(DR, mL))), inv);
    F[1] = mul2(fma2(dd, sub2(mR, mL), fma2(nDL, fr1, mul2(DR, fl1))), inv);
    F[2] = mul2(fma2(dd, fma2(rR, utR, mul2(mul2(rL, utL), pk(-1.0f, -1.0f))), fma2(nDL, fr2, mul2(DR, fl2))), inv);
    F[3] = mul2(fma2(dd, sub2(eR, eL), fma2(nDL, fr3, mul2(DR, fl3))), inv);
    // supersonic faces take one side's physical flux (rare: one branch for both)
    if (DL.x > 0.0f || DR.x < 0.0f || DL.y > 0.0f || DR.y < 0.0f) {
        if (DL.x > 0.0f) { F[0].x = mL.x; F[1].x = fl1.x; F[2].x = fl2.x; F[3].x = fl3.x; }
        else if (DR.x < 0.0f) { F[0].x = mR.x; F[1].x = fr1.x; F[2].x = fr2.x; F[3].x = fr3.x; }
        if (DL.y > 0.0f) { F[0].y = mL.y; F[1].y = fl1.y; F[2].y = fl2.y; F[3].y = fl3.y; }
        else if (DR.y < 0.0f) { F[0].y = mR.y; F[1].y = fr1.y; F[2].y = fr2.y; F[3].y = fr3.y; }
    }
}

// ------------------------------------------------------------------ HLLC (Aleksashov)
// The reference's second HLLC (HLLC_Aleksashov, kernel.cu:767-1079), an MHD
// HLLC solver it calls with zero magnetic field.  In the face frame (normal
// velocity un, tangential ut): fast speed sqrt(c c) (the B = 0 value of its
// fast-magnetosonic speed), Davis-type bounds, the contact speed SM and the
// star states with each side's own tangential velocity; the magnetic terms
// only add zeros.  The tangential flux is odd in ut, so one face-frame
// evaluation serves z faces (tangent +v_r) and r faces (the reference's
// tangent there is -v_z, its flux rotated back by the same sign).
template <typename R>
__device__ __forceinline__ R flux_hllc_a(const Gas<R>& g, R r1, R p1, R un1, R ut1, R r2, R p2, R un2, R ut2,
                                         R F[4])
{
    const R cL = sqrt(g.ga * p1 / r1), cR = sqrt(g.ga * p2 / r2);
    const R cfL = sqrt(cL * cL), cfR = sqrt(cR * cR);
    const R SL = fmin(un1 - cfL, un2 - cfR);
    const R SR = fmax(un1 + cfL, un2 + cfR);
    const R suR = SR - un2, suL = SL - un1;
    const R SM = (suR * r2 * un2 - p2 + p1 - suL * r1 * un1) / (suR * r2 - suL * r1);
    const R UU = fmax(fabs(SL), fabs(SR));
    const R e1 = p1 / g.g1 + r1 * ((un1 * un1 + ut1 * ut1) / R(2));
    const R e2 = p2 / g.g1 + r2 * ((un2 * un2 + ut2 * ut2) / R(2));
    // the reference's order of the four cases (SM can fall outside [SL, SR]
    // by rounding)
    if (SL > R(0)) {
        F[0] = r1 * un1; F[1] = r1 * un1 * un1 + p1; F[2] = r1 * un1 * ut1; F[3] = (e1 + p1) * un1;
    } else if (SM >= R(0)) {
        // left star state
        const R suLm = suL / (SL - SM), rz = r1 * suLm;
        const R ptz = ((p2 + r2 * suR * (SM - un2)) + (p1 + r1 * suL * (SM - un1))) / R(2);
        const R ez = e1 * suLm + (ptz * SM - p1 * un1) / (SL - SM);
        F[0] = r1 * un1 + SL * (rz - r1);
        F[1] = (r1 * un1 * un1 + p1) + SL * (SM * rz - r1 * un1);
        F[2] = r1 * un1 * ut1 + SL * (ut1 * rz - r1 * ut1);
        F[3] = (e1 + p1) * un1 + SL * (ez - e1);
    } else if (SR >= R(0)) {
        // right star state
        const R suRm = suR / (SR - SM), rz = r2 * suRm;
        const R ptz = ((p2 + r2 * suR * (SM - un2)) + (p1 + r1 * suL * (SM - un1))) / R(2);
        const R ez = e2 * suRm + (ptz * SM - p2 * un2) / (SR - SM);
        F[0] = r2 * un2 + SR * (rz - r2);
        F[1] = (r2 * un2 * un2 + p2) + SR * (SM * rz - r2 * un2);
        F[2] = r2 * un2 * ut2 + SR * (ut2 * rz - r2 * ut2);
        F[3] = (e2 + p2) * un2 + SR * (ez - e2);
    } else if (SR < R(0)) {
        F[0] = r2 * un2; F[1] = r2 * un2 * un2 + p2; F[2] = r2 * un2 * ut2; F[3] = (e2 + p2) * un2;
    } else {
        F[0] = F[1] = F[2] = F[3] = R(NAN);
    }
    return UU;
}

// ------------------------------------------------------------------ HLLC
template <typename R>
__device__ __forceinline__ R flux_hllc(const Gas<R>& g, R rL, R pL, R u1, R v1, R rR, R pR, R u2, R v2, R F[4])
{
    R cL = sqrt(g.ga * pL / rL);
    R cR = sqrt(g.ga * pR / rR);
    R mxc = fmax(cL, cR);
    R SL = fmin(u1, u2) - mxc;
    R SR = fmax(u1, u2) + mxc;
    R S = fmax(fabs(SL), fabs(SR));
    R eL = pL * g.inv_g1 + rL * (u1 * u1 + v1 * v1) * R(0.5);
    R eR = pR * g.inv_g1 + rR * (u2 * u2 + v2 * v2) * R(0.5);
    if (SL >= R(0)) {
        R m = rL * u1;
        F[0] = m; F[1] = m * u1 + pL; F[2] = m * v1; F[3] = (eL + pL) * u1;
        return S;
    }
    if (SR <= R(0)) {
        R m = rR * u2;
        F[0] = m; F[1] = m * u2 + pR; F[2] = m * v2; F[3] = (eR + pR) * u2;
        return S;
    }
    R suR = SR - u2, suL = SL - u1;
    R SM = (suR * rR * u2 - suL * rL * u1 - pR + pL) / (suR * rR - suL * rL);
    R ptz = (pR + rR * suR * (SM - u2) + pL + rL * suL * (SM - u1)) * R(0.5);
    if (SM >= R(0)) {
        // left star state (Gas_Dinamic.cu:1707, 1773, 1789-1795)
        R inv = R(1) / (SL - SM);
        R rs = rL * suL * inv;
        R es = eL * suL * inv + (ptz * SM - pL * u1) * inv;
        R m = rL * u1;
        F[0] = m + SL * (rs - rL);
        F[1] = m * u1 + pL + SL * (rs * SM - m);
        F[2] = m * v1 + SL * (rs * v1 - rL * v1);
        F[3] = (eL + pL) * u1 + SL * (es - eL);
    } else {
        R inv = R(1) / (SR - SM);
        R rs = rR * suR * inv;
        R es = eR * suR * inv + (ptz * SM - pR * u2) * inv;
        R m = rR * u2;
        F[0] = m + SR * (rs - rR);
        F[1] = m * u2 + pR + SR * (rs * SM - m);
        F[2] = m * v2 + SR * (rs * v2 - rR * v2);
        F[3] = (eR + pR) * u2 + SR * (es - eR);
    }
    return S;
}

// The passive-scalar flux of the HLLC solver above (the Q channel of
// HLLC_2d_Korolkov_b_s, Gas_Dinamic.cu:1660-1808, metod 2, W = 0): Q is a
// density carried by the flow, its flux Q u on the upwind side and, in a
// star region, the side's flux corrected by S (Q* - Q) with
// Q* = Q (S - u)/(S - SM).  The wave speeds and the contact speed are
// flux_hllc's, formed by the same expressions, so the scalar moves with
// that solver's mass flux.
template <typename R>
__device__ __forceinline__ R flux_hllc_q(const Gas<R>& g, R rL, R pL, R u1, R QL, R rR, R pR, R u2, R QR)
{
    R cL = sqrt(g.ga * pL / rL);
    R cR = sqrt(g.ga * pR / rR);
    R mxc = fmax(cL, cR);
    R SL = fmin(u1, u2) - mxc;
    R SR = fmax(u1, u2) + mxc;
    if (SL >= R(0)) return QL * u1;
    if (SR <= R(0)) return QR * u2;
    R suR = SR - u2, suL = SL - u1;
    R SM = (suR * rR * u2 - suL * rL * u1 - pR + pL) / (suR * rR - suL * rL);
    if (SM >= R(0)) {
        R inv = R(1) / (SL - SM);
        R qs = QL * suL * inv;
        return QL * u1 + SL * qs - SL * QL;
    }
    R inv = R(1) / (SR - SM);
    R qs = QR * suR * inv;
    return QR * u2 + SR * qs - SR * QR;
}

// ------------------------------------------------------------------ HLLC with a passive scalar (Korolkov)
// HLLCQ_Korolkov_2D (Gas_Dinamic.cu:249-353): an HLLC solver whose wave
// bounds are min(u_L - c_L, u_R - c_R) and max(u_L + c_L, u_R + c_R), with a
// passive scalar Q (a density: flux Q u upwind, Q rr/rho in a star region),
// in the face frame (normal un, tangential ut; each side's kinetic energy
// from its own components).  The tangential flux is odd in ut, so one
// evaluation serves z faces (tangent +v_r) and r faces (the reference's
// tangent there is -v_z, its flux rotated back by the same sign).  F = (mass,
// normal momentum, tangential momentum, energy), FQ the scalar's flux;
// returns max(|S_L|, |S_R|), whose dt candidate the reference forms as
// krit*rad/that.  Expression order as the reference's.
template <typename R>
__device__ __forceinline__ R flux_hllcq(const Gas<R>& g, R ro1, R p1, R u_L, R v_L, R Q_L, R ro2, R p2, R u_R, R v_R,
                                        R Q_R, R F[4], R& FQ)
{
    const R cL = sqrt(g.ga * p1 / ro1);
    const R cR = sqrt(g.ga * p2 / ro2);
    const R SL = fmin((u_L - cL), (u_R - cR));
    const R SR = fmax((u_L + cL), (u_R + cR));
    const R UU = fmax(fabs(SL), fabs(SR));
    const R FL1 = ro1 * u_L * u_L + p1;
    const R FL2 = ro1 * u_L * v_L;
    const R FR1 = ro2 * u_R * u_R + p2;
    const R FR2 = ro2 * u_R * v_R;
    if (SL >= R(0)) {
        FQ = Q_L * u_L;
        F[0] = ro1 * u_L;
        F[3] = (g.ga * p1 / (g.g1) + R(0.5) * ro1 * (u_L * u_L + v_L * v_L)) * u_L;
        F[1] = FL1;
        F[2] = FL2;
        return UU;
    }
    if (SR <= R(0)) {
        FQ = Q_R * u_R;
        F[0] = ro2 * u_R;
        F[3] = (g.ga * p2 / (g.g1) + R(0.5) * ro2 * (u_R * u_R + v_R * v_R)) * u_R;
        F[1] = FR1;
        F[2] = FR2;
        return UU;
    }
    const R SM = ((SR - u_R) * ro2 * u_R - (SL - u_L) * ro1 * u_L - p2 + p1) / ((SR - u_R) * ro2 - (SL - u_L) * ro1);
    const R pp = p1 + ro1 * (SL - u_L) * (SM - u_L);
    if (SM <= R(0)) {
        const R rr = ro2 * (SR - u_R) / (SR - SM);
        const R e = p2 / g.g1 + R(0.5) * ro2 * (u_R * u_R + v_R * v_R);
        const R ee = ((SR - u_R) * e - p2 * u_R + pp * SM) / (SR - SM);
        FQ = SR * (rr * Q_R / ro2 - Q_R) + Q_R * u_R;
        F[0] = SR * (rr - ro2) + ro2 * u_R;
        F[3] = SR * (ee - e) + (g.ga * p2 / (g.g1) + R(0.5) * ro2 * (u_R * u_R + v_R * v_R)) * u_R;
        F[1] = (ro2 * u_R * u_R + p2) + SR * (rr * SM - ro2 * u_R);
        F[2] = (ro2 * u_R * v_R) + SR * (rr * v_R - ro2 * v_R);
    } else if (SM >= R(0)) {
        const R rr = ro1 * (SL - u_L) / (SL - SM);
        const R e = p1 / g.g1 + R(0.5) * ro1 * (u_L * u_L + v_L * v_L);
        const R ee = ((SL - u_L) * e - p1 * u_L + pp * SM) / (SL - SM);
        FQ = SL * (rr * Q_L / ro1 - Q_L) + Q_L * u_L;
        F[0] = SL * (rr - ro1) + ro1 * u_L;
        F[3] = SL * (ee - e) + (g.ga * p1 / (g.g1) + R(0.5) * ro1 * (u_L * u_L + v_L * v_L)) * u_L;
        F[1] = FL1 + SL * (rr * SM - ro1 * u_L);
        F[2] = FL2 + SL * (rr * v_L - ro1 * v_L);
    } else {
        // SM is not a number (the reference prints an error and leaves the
        // flux unset): a non-finite flux, reported by the caller
        FQ = R(NAN);
        F[0] = F[1] = F[2] = F[3] = R(NAN);
    }
    return UU;
}

// ------------------------------------------------------------------ exact Riemann solver
// residual of the shock-rarefaction pattern (lev, kernel.cu:751-765)
template <typename R>
__device__ __forceinline__ R lev_res(const Gas<R>& g, R enI, R pI, R rI, R cI, R enII, R pII, R cII, R x)
{
    R fI = (x - pI) / (rI * cI * sqrt(g.gp * x / pI + g.gm));
    R fII = R(2) / g.g1 * cII * (pow(x / pII, g.gm) - R(1));
    return (fI + fII) - (enI - enII);
}

// bisection on [pI, pII] (devtwo, kernel.cu:682-749) with an iteration cap
template <typename R>
__device__ R bisect_p(const Gas<R>& g, R enI, R pI, R rI, R cI, R enII, R pII, R cII, RiemannCount& rc)
{
    R kl = pI, kp = pII;
    R ksi = lev_res(g, enI, pI, rI, cI, enII, pII, cII, kl);
    R ksir = lev_res(g, enI, pI, rI, cI, enII, pII, cII, kp);
    rc.bisect_calls++;
    if (fabs(ksi) <= g.tol) return kl;
    if (fabs(ksir) <= g.tol) return kp;
    R kc = kl;
    int it = 0;
    for (;;) {
        it++;
        kc = (kl + kp) / R(2);
        R ksit = lev_res(g, enI, pI, rI, cI, enII, pII, cII, kc);
        if (fabs(ksit) <= g.tol) break;
        if (it >= g.max_iter) { rc.status |= 0x08u; break; }
        if (ksi * ksit <= R(0)) { kp = kc; }
        else { kl = kc; ksi = ksit; }
    }
    rc.bisect_iters += it;
    return kc;
}

// Newton for the two-shock pattern (newton, kernel.cu:635-680) from start pn
template <typename R>
__device__ R newton_p(const Gas<R>& g, R enI, R pI, R rI, R cI, R enII, R pII, R rII, R cII, R pn,
                      RiemannCount& rc)
{
    const R pee = pn;
    const R aI = R(4) * g.ga * rI * cI, aII = R(4) * g.ga * rII * cII;
    const R b = R(3) * g.ga - R(1);
    int k = 0;
    R p;
    for (;;) {
        p = pn;
        k++;
        R qI = g.gp * p / pI + g.gm, qII = g.gp * p / pII + g.gm;
        R sI = sqrt(qI), sII = sqrt(qII);
        R fI = (p - pI) / (rI * cI * sI);
        R fII = (p - pII) / (rII * cII * sII);
        // pow(q, 3/2) = q*sqrt(q)
        R fIs = ((g.ga + R(1)) * p / pI + b) / (aI * qI * sI);
        R fIIs = ((g.ga + R(1)) * p / pII + b) / (aII * qII * sII);
        pn = p - (fI + fII - (enI - enII)) / (fIs + fIIs);
        if (!(fabs(pn / pee - p / pee) >= g.tol)) break;
        if (k >= g.max_iter) { rc.status |= 0x04u; break; }
    }
    rc.newton_calls++;
    rc.newton_iters += k;
    if (k > rc.newton_max) rc.newton_max = k;
    return pn;
}

// The exact Riemann problem of one face in the reference's frame, where
// the side with the lower pressure is side I (kernel.cu:144-184), with the
// wave-pattern thresholds of kernel.cu:186-231:
//   pattern 0  vacuum (Udf < Uvk)
//           1  two rarefactions (Uvk <= Udf <= Urz), p* in closed form
//           2  shock on side I, rarefaction on side II (Urz < Udf <= Uud),
//              p* in [pI, pII] (bisection in the reference)
//           3  two shocks (Udf > Uud), p* > pII (Newton in the reference)
//           4  no pattern (NaN input)
template <typename R>
struct RPre {
    R enI, teI, pI, rI, cI, enII, teII, pII, rII, cII;
    R Udf, Urz, Uvk;
    bool swap;
    int pattern;
};

// the side swap (pI <= pII, normal velocities negated when swapped) and the
// sound speeds of the two sides: the part of godunov_pre an iterative face
// needs again once its pattern is known
template <typename R>
__device__ __forceinline__ RPre<R> godunov_sides(const Gas<R>& g, R rL, R pL, R unL, R utL, R rR, R pR, R unR,
                                                 R utR)
{
    RPre<R> q;
    q.swap = pL > pR;
    if (q.swap) {
        q.enI = -unR; q.teI = utR; q.pI = pR; q.rI = rR;
        q.enII = -unL; q.teII = utL; q.pII = pL; q.rII = rL;
    } else {
        q.enI = unL; q.teI = utL; q.pI = pL; q.rI = rL;
        q.enII = unR; q.teII = utR; q.pII = pR; q.rII = rR;
    }
    q.cI = (q.rI != R(0)) ? sqrt(g.ga * q.pI / q.rI) : R(0);
    q.cII = (q.rII != R(0)) ? sqrt(g.ga * q.pII / q.rII) : R(0);
    q.Udf = q.enI - q.enII;
    q.Urz = q.Uvk = R(0);
    q.pattern = 4;
    return q;
}

template <typename R>
__device__ __forceinline__ RPre<R> godunov_pre(const Gas<R>& g, R rL, R pL, R unL, R utL, R rR, R pR, R unR,
                                               R utR)
{
    RPre<R> q = godunov_sides(g, rL, pL, unL, utL, rR, pR, unR, utR);
    const R a = sqrt(q.rI * (g.g2 * q.pII + g.g1 * q.pI) / R(2));
    const R Uud = (q.pII - q.pI) / a;
    if (q.Udf > R(0)) {
        // Uvk <= 0 and Urz <= 0 (pI <= pII, so (pI/pII)^gm <= 1): neither
        // vacuum nor two rarefactions, and only pattern 1 reads Urz and Uvk,
        // so the pow of Urz is not needed (same patterns as the full test)
        if (q.Udf <= Uud) q.pattern = 2;
        else if (q.Udf > Uud) q.pattern = 3;
        else q.pattern = 4;
        return q;
    }
    q.Urz = R(-2) * q.cII / g.g1 * (R(1) - pow(q.pI / q.pII, g.gm));
    q.Uvk = R(-2) * (q.cII + q.cI) / g.g1;
    if (q.Udf < q.Uvk) q.pattern = 0;
    else if (q.Udf <= q.Urz) q.pattern = 1;
    else if (q.Udf <= Uud) q.pattern = 2;
    else if (q.Udf > Uud) q.pattern = 3;
    else q.pattern = 4;
    return q;
}

// p* of patterns 2 and 3 as the reference finds it: bisection on [pI, pII]
// or Newton from the acoustic start value (kernel.cu:220-231, 641-642)
template <typename R>
__device__ __forceinline__ R solve_p_reference(const Gas<R>& g, const RPre<R>& q, RiemannCount& rc)
{
    if (q.pattern == 2) return bisect_p(g, q.enI, q.pI, q.rI, q.cI, q.enII, q.pII, q.cII, rc);
    const R p0 = (q.pI * q.rII * q.cII + q.pII * q.rI * q.cI + (q.enI - q.enII) * q.rI * q.cI * q.rII * q.cII) /
                 (q.rI * q.cI + q.rII * q.cII);
    return newton_p(g, q.enI, q.pI, q.rI, q.cI, q.enII, q.pII, q.rII, q.cII, p0, rc);
}

// The acoustic (PVRS-type) start value of the reference, kept inside the
// pattern's bracket: [pI, pII] for pattern 2, above pII for pattern 3.
template <typename R>
__device__ __forceinline__ R pvrs_guess(const RPre<R>& q)
{
    R p0 = (q.pI * q.rII * q.cII + q.pII * q.rI * q.cI + (q.enI - q.enII) * q.rI * q.cI * q.rII * q.cII) /
           (q.rI * q.cI + q.rII * q.cII);
    if (q.pattern == 2) p0 = fmin(fmax(p0, q.pI), q.pII);
    else p0 = fmax(p0, q.pII);
    return p0;
}

// true when p0 can start the safeguarded Newton iteration of the pattern:
// finite and inside the pattern's bracket widened by a factor 2 on each
// side (the pressure function is increasing and concave, and the iteration
// keeps the original bracket as its safeguard, so a start just outside it
// converges as fast as one just inside)
template <typename R>
__device__ __forceinline__ bool in_basin(const RPre<R>& q, R p0)
{
    if (!(p0 == p0) || !(p0 > R(0))) return false;
    if (q.pattern == 2) return p0 >= R(0.5) * q.pI && p0 <= R(2) * q.pII;
    return p0 >= R(0.5) * q.pII && p0 < R(1e30);
}

// convergence threshold of the relative Newton step: the requested
// tolerance, but not below 4 ulps of the arithmetic (1e-8 is below FP32
// resolution; the same clamp applies to every start value)
template <typename R>
__device__ __forceinline__ R newton_tol(R tol);
template <>
__device__ __forceinline__ double newton_tol<double>(double tol) { return tol; }
template <>
__device__ __forceinline__ float newton_tol<float>(float tol) { return fmaxf(tol, 4.0f * 1.1920929e-7f); }

// Safeguarded Newton on the full pressure function
//   f(p) = f_I(p) + f_II(p) - (enI - enII),
// f_K the shock branch (kernel.cu:656-662) for p > p_K and the rarefaction
// branch (lev, kernel.cu:759) for p <= p_K, from start value p0 to the
// relative change tol.  The bracket of the root ([pI, pII] or (pII, inf))
// shrinks with the sign of f; an iterate that leaves it is replaced by the
// bracket's upper edge (or, below it, by a bisection step).
template <typename R>
__device__ R solve_p_newton(const Gas<R>& g, const RPre<R>& q, R p0, R tol, RiemannCount& rc)
{
    R lo = (q.pattern == 2) ? q.pI : q.pII;
    R hi = (q.pattern == 2) ? q.pII : R(INFINITY);
    const R dU = q.enI - q.enII;
    const R b = R(3) * g.ga - R(1);
    R p = p0;
    R prev_step = R(INFINITY);
    int k = 0;
    for (;;) {
        k++;
        R f = -dU, df = R(0);
#pragma unroll
        for (int side = 0; side < 2; side++) {
            const R pK = side ? q.pII : q.pI, rK = side ? q.rII : q.rI, cK = side ? q.cII : q.cI;
            if (p > pK) {
                const R qq = g.gp * p / pK + g.gm, sq = sqrt(qq);
                f += (p - pK) / (rK * cK * sq);
                df += ((g.ga + R(1)) * p / pK + b) / (R(4) * g.ga * rK * cK * qq * sq);
            } else {
                const R t = pow(p / pK, g.gm);
                f += R(2) / g.g1 * cK * (t - R(1));
                df += t / (rK * cK) * (pK / p);
            }
        }
        if (f < R(0)) lo = fmax(lo, p); else hi = fmin(hi, p);
        R pn = p - f / df;
        // converged: tested before the bracket, since at convergence the step
        // may round onto the bracket's edge
        if (fabs(pn - p) <= newton_tol(tol) * p) {
            p = pn;
            break;
        }
        // f is increasing and concave: from f < 0 a Newton step overshoots
        // the root; an overshoot past the bracket restarts from its upper
        // edge, from where the iteration descends monotonically
        if (!(pn > lo && pn < hi)) pn = (pn >= hi) ? hi : R(0.5) * (lo + fmin(hi, R(2) * p));
        const R step = fabs(pn - p);
        // a step no shorter than the previous one: the iteration has reached
        // the rounding noise of f
        const bool done = k > 2 && step >= prev_step;
        prev_step = step;
        p = pn;
        if (done) break;
        if (k >= g.max_iter) { rc.status |= 0x04u; break; }
    }
    rc.newton_calls++;
    rc.newton_iters += k;
    if (k > rc.newton_max) rc.newton_max = k;
    return p;
}

// Mass-flux coefficient of a rarefaction, g_m rho c (1 - x)/(1 - x^g_m) with
// x = p/p_K, as the reference forms it (kernel.cu:297-304, 371-389): the
// limit rho c when |p - p_K| < eps.  In FP32 the quotient cancels
// catastrophically near x = 1, so there the three-term series in d = 1 - x
// (d/(1-(1-d)^g) expanded about d = 0) is used for |d| < 0.02.
template <typename R>
__device__ __forceinline__ R rare_coef(const Gas<R>& g, R rK, R cK, R p, R pK)
{
    return (fabs(p - pK) < g.eps) ? rK * cK : g.gm * rK * cK * (R(1) - p / pK) / (R(1) - pow(p / pK, g.gm));
}

template <>
__device__ __forceinline__ float rare_coef<float>(const Gas<float>& g, float rK, float cK, float p, float pK)
{
    const float d = 1.0f - p / pK;
    if (fabsf(d) < 0.02f) {
        const float a = 0.5f * (g.gm - 1.0f);
        const float b = (g.gm - 1.0f) * (g.gm - 2.0f) * (1.0f / 6.0f);
        const float c = (g.gm - 1.0f) * (g.gm - 2.0f) * (g.gm - 3.0f) * (1.0f / 24.0f);
        return rK * cK * (1.0f + d * (a + d * ((a * a - b) + d * (a * a * a - 2.0f * a * b + c))));
    }
    return g.gm * rK * cK * d / (1.0f - powf(1.0f - d, g.gm));
}

// Sampling of the solution at w = 0 and the face flux (kernel.cu:233-568).
// p: the solved p* for patterns 2 and 3 (ignored otherwise).  Returns the dt
// wave speed max(UU, eps8), UU the largest wave speed of the pattern.
// MODE: every pattern (kSampleAll), or only the closed-form patterns 0 and 1
// (kSampleClosed) or the iterative ones 2 and 3 (kSampleIterative) for a
// caller that has sorted its faces by pattern (the other patterns' code is
// left out of that caller; a face of another pattern samples as NaN)
enum { kSampleAll = 0, kSampleClosed = 1, kSampleIterative = 2 };
template <typename R, int MODE = kSampleAll>
__device__ R godunov_sample(const Gas<R>& g, const RPre<R>& q, R p, R F[4], RiemannCount& rc)
{
    const R enI = q.enI, teI = q.teI, pI = q.pI, rI = q.rI, cI = q.cI;
    const R enII = q.enII, teII = q.teII, pII = q.pII, rII = q.rII, cII = q.cII;
    R en, r, te, UU;
    // The reference tests the fan intervals with independent ifs
    // (kernel.cu:322-363, 419-476, 502-543), so a later interval overrides
    // an earlier one; the same order is kept here.
    const R w = R(0);
    en = r = te = UU = R(0);
    if (MODE != kSampleIterative && q.pattern == 0) {
        // vacuum between two rarefactions
        rc.status |= 0x20u;
        p = R(0);
        R dI = enI - cI, ddI = enI + R(2) / g.g1 * cI;
        R dII = enII + cII, ddII = enII - R(2) / g.g1 * cII;
        UU = fmax(fmax(fabs(dI), fabs(dII)), fmax(fabs(ddII), fabs(ddI)));
        if (w <= dI) { en = enI; p = pI; r = rI; te = teI; }
        if ((w > dI) && (w < ddI)) {
            R ce = g.g1 / g.g2 * (enI - w) + R(2) / g.g2 * cI;
            en = w + ce; p = pI * pow(ce / cI, R(1) / g.gm); r = g.ga * p / ce / ce; te = teI;
        }
        if ((w >= ddI) && (w <= ddII)) { en = w; p = R(0); r = R(0); te = R(0); }
        if ((w > ddII) && (w < dII)) {
            R ce = -g.g1 / g.g2 * (enII - w) + R(2) / g.g2 * cII;
            en = w - ce; p = pII * pow(ce / cII, R(1) / g.gm); r = g.ga * p / ce / ce; te = teII;
        }
        if (w >= dII) { en = enII; p = pII; r = rII; te = teII; }
    } else if (MODE != kSampleIterative && q.pattern == 1) {
        // two rarefactions, closed form
        p = pI * pow((q.Udf - q.Uvk) / (q.Urz - q.Uvk), R(1) / g.gm);
        R aI = rare_coef(g, rI, cI, p, pI);
        R aII = rare_coef(g, rII, cII, p, pII);
        R u = (aI * enI + aII * enII + pI - pII) / (aI + aII);
        R dI = enI - cI;
        R ddI = u - cI - g.g1 * (enI - u) / R(2);
        R dII = enII + cII;
        R ddII = u + cII - g.g1 * (enII - u) / R(2);
        UU = fmax(fmax(fabs(dI), fabs(dII)), fmax(fabs(ddII), fabs(ddI)));
        if (w <= dI) { en = enI; p = pI; r = rI; te = teI; }
        if ((w > dI) && (w < ddI)) {
            R ce = g.g1 / g.g2 * (enI - w) + R(2) / g.g2 * cI;
            en = w + ce; p = pI * pow(ce / cI, R(1) / g.gm); r = g.ga * p / ce / ce; te = teI;
        }
        if ((w >= ddI) && (w <= u)) {
            R ce = cI + g.g1 / R(2) * (enI - u);
            en = u; r = g.ga * p / ce / ce; te = teI;
        }
        if ((w > u) && (w <= ddII)) {
            R ce = cII - g.g1 / R(2) * (enII - u);
            en = u; r = g.ga * p / ce / ce; te = teII;
        }
        if ((w > ddII) && (w < dII)) {
            R ce = -g.g1 / g.g2 * (enII - w) + R(2) / g.g2 * cII;
            en = w - ce; p = pII * pow(ce / cII, R(1) / g.gm); r = g.ga * p / ce / ce; te = teII;
        }
        if (w >= dII) { en = enII; p = pII; r = rII; te = teII; }
    } else if (MODE != kSampleClosed && q.pattern == 2) {
        // shock on side I, rarefaction on side II
        R aI = sqrt(rI * (g.g2 / R(2) * p + g.g1 / R(2) * pI));
        R aII = rare_coef(g, rII, cII, p, pII);
        R u = (aI * enI + aII * enII + pI - pII) / (aI + aII);
        R dI = enI - aI / rI;
        R dII = enII + cII;
        R ddII = u + cII - g.g1 * (enII - u) / R(2);
        UU = fmax(fmax(fabs(dI), fabs(dII)), fabs(ddII));
        if (w <= dI) { en = enI; p = pI; r = rI; te = teI; }
        if ((w > dI) && (w <= u)) { en = u; r = rI * aI / (aI - rI * (enI - u)); te = teI; }
        if ((w > u) && (w <= ddII)) {
            R ce = cII - g.g1 / R(2) * (enII - u);
            en = u; r = g.ga * p / ce / ce; te = teII;
        }
        if ((w > ddII) && (w < dII)) {
            R ce = -g.g1 / g.g2 * (enII - w) + R(2) / g.g2 * cII;
            en = w - ce; p = pII * pow(ce / cII, R(1) / g.gm); r = g.ga * p / ce / ce; te = teII;
        }
        if (w >= dII) { en = enII; p = pII; r = rII; te = teII; }
    } else if (MODE != kSampleClosed && q.pattern == 3) {
        // two shocks
        R aI = sqrt(rI * (g.g2 / R(2) * p + g.g1 / R(2) * pI));
        R aII = sqrt(rII * (g.g2 / R(2) * p + g.g1 / R(2) * pII));
        R u = (aI * enI + aII * enII + pI - pII) / (aI + aII);
        R dI = enI - aI / rI;
        R dII = enII + aII / rII;
        UU = fmax(fabs(dI), fabs(dII));
        if (w <= dI) { en = enI; p = pI; r = rI; te = teI; }
        else if (w <= u) { en = u; r = rI * aI / (aI - rI * (enI - u)); te = teI; }
        else if (w < dII) { en = u; r = rII * aII / (aII + rII * (enII - u)); te = teII; }
        else { en = enII; p = pII; r = rII; te = teII; }
    } else {
        rc.status |= 0x10u;
        en = p = r = te = UU = R(NAN);
    }
    if (q.swap) en = -en;
    R e = p * g.inv_g1 + R(0.5) * r * (en * en + te * te);
    R m = r * en;
    F[0] = m;
    F[1] = m * en + p;
    F[2] = m * te;
    F[3] = en * (e + p);
    return (UU > g.eps8) ? UU : g.eps8;
}

// Exact Godunov flux of one face with the reference's solver
// (Godunov_Solver_Alexashov, kernel.cu:128-570).
template <typename R>
__device__ R flux_godunov(const Gas<R>& g, R rL, R pL, R unL, R utL, R rR, R pR, R unR, R utR, R F[4],
                          RiemannCount& rc)
{
    const RPre<R> q = godunov_pre(g, rL, pL, unL, utL, rR, pR, unR, utR);
    R p = R(0);
    if (q.pattern == 2 || q.pattern == 3) p = solve_p_reference(g, q, rc);
    return godunov_sample(g, q, p, F, rc);
}

}  // namespace ast
