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
    unsigned status;
    __device__ void clear() { newton_calls = newton_iters = bisect_calls = bisect_iters = newton_max = 0; status = 0; }
};

// ------------------------------------------------------------------ minmod
template <typename R>
__device__ __forceinline__ R minmod_d(R a, R b)
{
    // (sign a + sign b)/2 * min(|a|, |b|): zero unless both have one sign
    R m = fmin(fabs(a), fabs(b));
    return (a > R(0) && b > R(0)) ? m : ((a < R(0) && b < R(0)) ? -m : R(0));
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
    R mxc = fmax(cL, cR);
    R DL = fmin(unL, unR) - mxc;
    R DR = fmax(unL, unR) + mxc;
    R S = fmax(fabs(DL), fabs(DR));
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

// Exact Godunov flux, sampled at w = 0 (Godunov_Solver_Alexashov,
// kernel.cu:128-570).  Returns the dt wave speed: max(UU, eps8) with UU the
// largest wave speed magnitude of the pattern.
template <typename R>
__device__ R flux_godunov(const Gas<R>& g, R rL, R pL, R unL, R utL, R rR, R pR, R unR, R utR, R F[4],
                          RiemannCount& rc)
{
    R enI = unL, teI = utL, enII = unR, teII = utR;
    R pI = pL, pII = pR, rI = rL, rII = rR;
    const bool swap = pI > pII;
    if (swap) {
        enI = -unR; teI = utR; pI = pR; rI = rR;
        enII = -unL; teII = utL; pII = pL; rII = rL;
    }
    R cI = (rI != R(0)) ? sqrt(g.ga * pI / rI) : R(0);
    R cII = (rII != R(0)) ? sqrt(g.ga * pII / rII) : R(0);
    R a = sqrt(rI * (g.g2 * pII + g.g1 * pI) / R(2));
    R Uud = (pII - pI) / a;
    R Urz = R(-2) * cII / g.g1 * (R(1) - pow(pI / pII, g.gm));
    R Uvk = R(-2) * (cII + cI) / g.g1;
    R Udf = enI - enII;
    R en, p, r, te, UU;
    // Sampling at w = 0.  The reference tests the fan intervals with
    // independent ifs (kernel.cu:322-363, 419-476, 502-543), so a later
    // interval overrides an earlier one; the same order is kept here.
    const R w = R(0);
    en = p = r = te = UU = R(0);
    if (Udf < Uvk) {
        // vacuum between two rarefactions
        rc.status |= 0x20u;
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
    } else if (Udf <= Urz) {
        // two rarefactions, closed form
        p = pI * pow((Udf - Uvk) / (Urz - Uvk), R(1) / g.gm);
        R aI = (fabs(p - pI) < g.eps) ? rI * cI : g.gm * rI * cI * (R(1) - p / pI) / (R(1) - pow(p / pI, g.gm));
        R aII = (fabs(p - pII) < g.eps) ? rII * cII
                                        : g.gm * rII * cII * (R(1) - p / pII) / (R(1) - pow(p / pII, g.gm));
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
    } else if (Udf <= Uud) {
        // left shock, right rarefaction
        p = bisect_p(g, enI, pI, rI, cI, enII, pII, cII, rc);
        R aI = sqrt(rI * (g.g2 / R(2) * p + g.g1 / R(2) * pI));
        R aII = (fabs(p - pII) < g.eps) ? rII * cII
                                        : g.gm * rII * cII * (R(1) - p / pII) / (R(1) - pow(p / pII, g.gm));
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
    } else if (Udf > Uud) {
        // two shocks; acoustic start value (kernel.cu:641-642)
        R p0 = (pI * rII * cII + pII * rI * cI + (enI - enII) * rI * cI * rII * cII) / (rI * cI + rII * cII);
        p = newton_p(g, enI, pI, rI, cI, enII, pII, rII, cII, p0, rc);
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
        // NaN input: no pattern
        rc.status |= 0x10u;
        en = p = r = te = UU = R(NAN);
    }
    if (swap) en = -en;
    R e = p * g.inv_g1 + R(0.5) * r * (en * en + te * te);
    R m = r * en;
    F[0] = m;
    F[1] = m * en + p;
    F[2] = m * te;
    F[3] = en * (e + p);
    return (UU > g.eps8) ? UU : g.eps8;
}

}  // namespace ast
