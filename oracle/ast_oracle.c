/*
 * ast_oracle.c - CPU oracle for the explicit r-z finite-volume step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: the tests, the
 * smoke check and the CPU-baseline leg of the benchmark call it to produce
 * the expected answer.  The product (the CUDA library under
 * asteriy_2d_gb300/) never links, loads or calls it, and has no CPU path.
 *
 * It restates, in plain C, the algorithm of the reference's step kernels,
 * one cell at a time exactly as the reference threads do (each cell
 * evaluates its own four faces), with the same floating-point expression
 * order, so that it can be pinned bit-for-bit against the reference's own
 * functions compiled for the host (oracle/ref_driver.cpp) and against the
 * golden vectors generated from them (tests/golden/).
 *
 *   minmod / linear / linear2 ...... kernel.cu:22-50, sign Gas_Dinamic.cu:858-872
 *   HLL ............................ kernel.cu:1399-1523
 *   HLLC (Korolkov, metod 2, W=0) .. Gas_Dinamic.cu:1604-1826, with its
 *                                    passive-scalar channel (PQ)
 *   HLLCQ (Korolkov) ............... Gas_Dinamic.cu:249-353
 *   passive scalar step ............ not in the reference (its steps do not
 *                                    carry Q): the density's update form
 *                                    with the solvers' PQ, as the library
 *                                    carries it
 *   HLLC (Aleksashov, B = 0) ....... kernel.cu:767-1079
 *   exact Godunov .................. kernel.cu:128-570, newton :635-680,
 *                                    devtwo :682-749, lev :751-765
 *   stencil + ghost rules .......... kernel.cu:2549-2698 (Kernel_TVD),
 *                                    kernel.cu:2328-2382 (add_MK)
 *   reconstruction + faces ......... kernel.cu:2701-2857
 *   planar update .................. kernel.cu:3027-3073
 *   axisymmetric update ............ kernel.cu:2480-2509, with add_MK's
 *                                    neutral-coupling momentum source
 *                                    (nn2, kernel.cu:2495-2496; also applied
 *                                    to the planar update when set)
 *   dt (exact min, lagged) ......... kernel.cu:3013-3017, funk_time :1525-1536
 *   characteristic inflow .......... add2_bound kernel.cu:1895-1925
 *   non-reflecting ghost ........... the commented rule of add2, kernel.cu:1979-1985
 *                                    (restated from the comment: the reference
 *                                    compiles no code for it, so it is not pinned)
 *
 * Differences from the reference, all deliberate:
 *   - gamma, CFL, grid, boundaries, flux and tolerances are runtime values;
 *   - the dt minimum is exact (the reference's global write races);
 *   - Newton and bisection stop after riemann_max_iter iterations (the
 *     reference loops without bound) and count that event.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -shared -fPIC (see
 * oracle/build_oracle.py).  -ffp-contract=off keeps every multiply and add
 * separately rounded, as the reference's expressions are written.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/asteriy_gb300.h"

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double x, y; } d2;

/* counters of one step (summed over cells) */
typedef struct ora_stats {
    int64_t rho_floor, p_floor;
    int64_t newton_calls, newton_iters, newton_cap;
    int64_t bisect_calls, bisect_iters, bisect_cap;
    int64_t vacuum;
    int64_t newton_max;
    /* smallest | |residual| - tol | / tol over the bisection's stopping
       tests since the cell began (the per-cell margin diagnostic) */
    double margin;
    /* smallest distance of Udf to a wave-pattern threshold (Uvk, Urz,
       Uud), relative to cI + cII, over the faces with unequal states */
    double pmargin;
} ora_stats;

/* physical constants of one configuration (Header.h:17-26, 47, 62-63) */
typedef struct ora_phys {
    double ga, g1, g2, gp, gm;   /* gamma, gamma-1, gamma+1, (g2/ga)/2, (g1/ga)/2 */
    double krit;                 /* CFL number                                  */
    double eps;                  /* Newton / bisection tolerance                */
    double eps8;                 /* 10e-8: smallest wave speed used for dt      */
    int max_iter;
} ora_phys;

static void ora_phys_init(ora_phys* ph, double gamma, double krit, double tol, int max_iter)
{
    ph->ga = gamma;
    ph->g1 = gamma - 1.0;
    ph->g2 = gamma + 1.0;
    ph->gp = (ph->g2 / ph->ga) / 2.0;
    ph->gm = (ph->g1 / ph->ga) / 2.0;
    ph->krit = krit;
    ph->eps = tol;
    ph->eps8 = 10e-8;
    ph->max_iter = max_iter;
}

/* ------------------------------------------------------------------------ */
/* reconstruction (kernel.cu:22-50)                                          */
/* ------------------------------------------------------------------------ */
static int ora_sign(double x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); }

double ora_minmod(double a, double b)
{
    int s = ora_sign(a) + ora_sign(b);
    if (s == 0) return 0.0;
    return (s / 2.0) * fmin(fabs(a), fabs(b));
}

double ora_linear(double x1, double t1, double x2, double t2, double x3, double t3, double y)
{
    double d = ora_minmod((t1 - t2) / (x1 - x2), (t2 - t3) / (x2 - x3));
    return d * (y - x2) + t2;
}

void ora_linear2(double x1, double t1, double x2, double t2, double x3, double t3,
                 double y1, double y2, double* A, double* B)
{
    double d = ora_minmod((t1 - t2) / (x1 - x2), (t2 - t3) / (x2 - x3));
    *A = d * (y1 - x2) + t2;
    *B = d * (y2 - x2) + t2;
}

/* ------------------------------------------------------------------------ */
/* HLL (kernel.cu:1399-1523).  Ps = (mass, energy), Pu = (mom_z, mom_r).     */
/* ------------------------------------------------------------------------ */
static double hll(const ora_phys* ph, d2 Ls, d2 Lu, d2 Rs, d2 Ru, double n1, double n2,
                  d2* Ps, d2* Pu, double rad)
{
    const double ggg = ph->ga;
    double ro_L = Ls.x, p_L = Ls.y, v1_L = Lu.x, v2_L = Lu.y;
    double ro_R = Rs.x, p_R = Rs.y, v1_R = Ru.x, v2_R = Ru.y;
    double Vkv_L = v1_L * v1_L + v2_L * v2_L;
    double Vkv_R = v1_R * v1_R + v2_R * v2_R;
    double c_L = (ro_L <= 0) ? 0.0 : sqrt(ggg * p_L / ro_L);
    double c_R = (ro_R <= 0) ? 0.0 : sqrt(ggg * p_R / ro_R);
    double e_L = p_L / (ggg - 1.0) + ro_L * Vkv_L / 2.0;
    double e_R = p_R / (ggg - 1.0) + ro_R * Vkv_R / 2.0;
    double Vn_L = v1_L * n1 + v2_L * n2;
    double Vn_R = v1_R * n1 + v2_R * n2;
    double mnV = (Vn_L <= Vn_R) ? Vn_L : Vn_R;
    double mxV = (Vn_L >= Vn_R) ? Vn_L : Vn_R;
    double mxc = (c_L >= c_R) ? c_L : c_R;
    double D_L = mnV - mxc;
    double D_R = mxV + mxc;
    double aL = fabs(D_L), aR = fabs(D_R);
    double den = (aL >= aR) ? aL : aR;
    double t = 10000000;
    double tc = ph->krit * rad / den;
    t = (t <= tc) ? t : tc;

    double fx1 = ro_L * v1_L, fx2 = ro_L * v1_L * v1_L + p_L, fx3 = ro_L * v1_L * v2_L, fx5 = (e_L + p_L) * v1_L;
    double fy1 = ro_L * v2_L, fy2 = ro_L * v1_L * v2_L, fy3 = ro_L * v2_L * v2_L + p_L, fy5 = (e_L + p_L) * v2_L;
    double fl_1 = fx1 * n1 + fy1 * n2, fl_2 = fx2 * n1 + fy2 * n2;
    double fl_3 = fx3 * n1 + fy3 * n2, fl_5 = fx5 * n1 + fy5 * n2;
    if (D_L > 0.0) {
        Ps->x = fl_1; Pu->x = fl_2; Pu->y = fl_3; Ps->y = fl_5;
        return t;
    }
    double hx1 = ro_R * v1_R, hx2 = ro_R * v1_R * v1_R + p_R, hx3 = ro_R * v1_R * v2_R, hx5 = (e_R + p_R) * v1_R;
    double hy1 = ro_R * v2_R, hy2 = ro_R * v1_R * v2_R, hy3 = ro_R * v2_R * v2_R + p_R, hy5 = (e_R + p_R) * v2_R;
    double fr_1 = hx1 * n1 + hy1 * n2, fr_2 = hx2 * n1 + hy2 * n2;
    double fr_3 = hx3 * n1 + hy3 * n2, fr_5 = hx5 * n1 + hy5 * n2;
    if (D_R < 0.0) {
        Ps->x = fr_1; Pu->x = fr_2; Pu->y = fr_3; Ps->y = fr_5;
        return t;
    }
    double dq1 = ro_R - ro_L;
    double dq2 = ro_R * v1_R - ro_L * v1_L;
    double dq3 = ro_R * v2_R - ro_L * v2_L;
    double dq5 = e_R - e_L;
    Ps->x = (D_R * fl_1 - D_L * fr_1 + D_L * D_R * dq1) / (D_R - D_L);
    Pu->x = (D_R * fl_2 - D_L * fr_2 + D_L * D_R * dq2) / (D_R - D_L);
    Pu->y = (D_R * fl_3 - D_L * fr_3 + D_L * D_R * dq3) / (D_R - D_L);
    Ps->y = (D_R * fl_5 - D_L * fr_5 + D_L * D_R * dq5) / (D_R - D_L);
    return t;
}

/* ------------------------------------------------------------------------ */
/* HLLC, HLLC_2d_Korolkov_b_s with metod=2, W=0 (Gas_Dinamic.cu:1604-1826). */
/* The passive scalar Q does not feed the other outputs; its flux goes to   */
/* *PQ when PQ is not NULL (Q_L, Q_R its values on the two sides).          */
/* ------------------------------------------------------------------------ */
static double hllc_q(const ora_phys* ph, d2 Ls, d2 Lu, d2 Rs, d2 Ru, double Q_L, double Q_R, double n1,
                     double n2, d2* Ps, d2* Pu, double* PQ, double rad, int nul_potok)
{
    const double ggg = ph->ga, g1 = ph->g1, W = 0.0;
    double ro_L = Ls.x, p_L = Ls.y, v1_L = Lu.x, v2_L = Lu.y;
    double ro_R = Rs.x, p_R = Rs.y, v1_R = Ru.x, v2_R = Ru.y;
    double t1 = n2, t2 = -n1;
    double u1 = v1_L * n1 + v2_L * n2;
    double v1 = v1_L * t1 + v2_L * t2;
    double u2 = v1_R * n1 + v2_R * n2;
    double v2 = v1_R * t1 + v2_R * t2;
    double cL = sqrt(ggg * p_L / ro_L);
    double cR = sqrt(ggg * p_R / ro_R);
    double uu_L = (v1_L * v1_L + v2_L * v2_L) / 2.0;
    double uu_R = (v1_R * v1_R + v2_R * v2_R) / 2.0;
    double SL = fmin(u1, u2) - fmax(cL, cR);
    double SR = fmax(u1, u2) + fmax(cL, cR);
    double suR = (SR - u2);
    double suL = (SL - u1);
    double SM = (suR * ro_R * u2 - suL * ro_L * u1 - p_R + p_L) / (suR * ro_R - suL * ro_L);
    double UU = fmax(fabs(SL), fabs(SR));
    double time = ph->krit * rad / UU;
    double FL[4], FR[4], UL[4], UR[4], P[4];
    double e1 = p_L / g1 + ro_L * uu_L;
    double e2 = p_R / g1 + ro_R * uu_R;
    FL[0] = ro_L * u1; FL[1] = ro_L * u1 * u1 + p_L; FL[2] = ro_L * u1 * v1; FL[3] = (e1 + p_L) * u1;
    FR[0] = ro_R * u2; FR[1] = ro_R * u2 * u2 + p_R; FR[2] = ro_R * u2 * v2; FR[3] = (e2 + p_R) * u2;
    UL[0] = ro_L; UL[1] = ro_L * u1; UL[2] = ro_L * v1; UL[3] = e1;
    UR[0] = ro_R; UR[1] = ro_R * u2; UR[2] = ro_R * v2; UR[3] = e2;
    /* the scalar's column (index 4 of the reference's arrays) */
    double FL4 = Q_L * u1, FR4 = Q_R * u2, UL4 = Q_L, UR4 = Q_R, PQ4;

    if (SL >= W) {
        P[1] = n1 * (FL[1] - W * UL[1]) + t1 * (FL[2] - W * UL[2]);
        P[2] = n2 * (FL[1] - W * UL[1]) + t2 * (FL[2] - W * UL[2]);
        P[0] = FL[0] - W * UL[0];
        P[3] = FL[3] - W * UL[3];
        PQ4 = FL4 - W * UL4;
    } else if (SR <= W) {
        P[1] = n1 * (FR[1] - W * UR[1]) + t1 * (FR[2] - W * UR[2]);
        P[2] = n2 * (FR[1] - W * UR[1]) + t2 * (FR[2] - W * UR[2]);
        P[0] = FR[0] - W * UR[0];
        P[3] = FR[3] - W * UR[3];
        PQ4 = FR4 - W * UR4;
    } else {
        double ro_LL = ro_L * (SL - u1) / (SL - SM);
        double ro_RR = ro_R * (SR - u2) / (SR - SM);
        double Q_LL = Q_L * (SL - u1) / (SL - SM);
        double Q_RR = Q_R * (SR - u2) / (SR - SM);
        double suRm = suR / (SR - SM);
        double suLm = suL / (SL - SM);
        double ptzR = p_R + ro_R * suR * (SM - u2);
        double ptzL = p_L + ro_L * suL * (SM - u1);
        double ptz = (ptzR + ptzL) / 2.0;
        double vLL, vRR;
        if (nul_potok) {
            double UZ0 = (SR * UR[0] - SL * UL[0] + FL[0] - FR[0]) / (SR - SL);
            double UZ2 = (SR * UR[2] - SL * UL[2] + FL[2] - FR[2]) / (SR - SL);
            vRR = UZ2 / UZ0;
            vLL = vRR;
        } else {
            vLL = v1;
            vRR = v2;
        }
        double ee2 = e2 * suRm + (ptz * SM - p_R * u2) / (SR - SM);
        double ee1 = e1 * suLm + (ptz * SM - p_L * u1) / (SL - SM);
        double ULL[4], URR[4], PO[4];
        ULL[0] = ro_LL; ULL[1] = ro_LL * SM; ULL[2] = ro_LL * vLL; ULL[3] = ee1;
        URR[0] = ro_RR; URR[1] = ro_RR * SM; URR[2] = ro_RR * vRR; URR[3] = ee2;
        if (SL < W && SM >= W) {
            for (int i = 0; i < 4; i++) PO[i] = FL[i] + SL * ULL[i] - SL * UL[i] - W * ULL[i];
            PQ4 = FL4 + SL * Q_LL - SL * UL4 - W * Q_LL;
        } else if (SR > W && SM < W) {
            for (int i = 0; i < 4; i++) PO[i] = FR[i] + SR * URR[i] - SR * UR[i] - W * URR[i];
            PQ4 = FR4 + SR * Q_RR - SR * UR4 - W * Q_RR;
        } else {
            for (int i = 0; i < 4; i++) PO[i] = NAN;
            PQ4 = NAN;
        }
        P[1] = n1 * PO[1] + t1 * PO[2];
        P[2] = n2 * PO[1] + t2 * PO[2];
        P[0] = PO[0];
        P[3] = PO[3];
    }
    Ps->x = P[0]; Ps->y = P[3]; Pu->x = P[1]; Pu->y = P[2];
    if (PQ) *PQ = PQ4;
    return time;
}

static double hllc(const ora_phys* ph, d2 Ls, d2 Lu, d2 Rs, d2 Ru, double n1, double n2,
                   d2* Ps, d2* Pu, double rad, int nul_potok)
{
    return hllc_q(ph, Ls, Lu, Rs, Ru, 1.0, 1.0, n1, n2, Ps, Pu, NULL, rad, nul_potok);
}

/* ------------------------------------------------------------------------ */
/* HLLCQ_Korolkov_2D (Gas_Dinamic.cu:249-353): HLLC with the bounds         */
/* min(u_L - c_L, u_R - c_R), max(u_L + c_L, u_R + c_R) and the passive     */
/* scalar Q; tangent t = (-n2, n1).  A non-number contact speed leaves the  */
/* reference's outputs unset: NaN here.                                     */
/* ------------------------------------------------------------------------ */
static double hllcq(const ora_phys* ph, d2 Ls, d2 Lu, d2 Rs, d2 Ru, double LQ, double RQ, double n1, double n2,
                    d2* Ps, d2* Pu, double* PQ, double rad)
{
    const double ga = ph->ga, g1 = ph->g1;
    double ro1 = Ls.x, u1 = Lu.x, v1 = Lu.y, p1 = Ls.y, Q_L = LQ;
    double ro2 = Rs.x, u2 = Ru.x, v2 = Ru.y, p2 = Rs.y, Q_R = RQ;
    double t1 = -n2, t2 = n1;
    double u_L = u1 * n1 + v1 * n2;
    double v_L = u1 * t1 + v1 * t2;
    double u_R = u2 * n1 + v2 * n2;
    double v_R = u2 * t1 + v2 * t2;
    double cL = sqrt(ga * p1 / ro1);
    double cR = sqrt(ga * p2 / ro2);
    double SL = fmin((u_L - cL), (u_R - cR));
    double SR = fmax((u_L + cL), (u_R + cR));
    double UU = fmax(fabs(SL), fabs(SR));
    double time = ph->krit * rad / UU;
    double FL1 = ro1 * u_L * u_L + p1;
    double FL2 = ro1 * u_L * v_L;
    double FR1 = ro2 * u_R * u_R + p2;
    double FR2 = ro2 * u_R * v_R;
    double q;
    if (SL >= 0.0) {
        q = Q_L * u_L;
        Ps->x = ro1 * u_L;
        Ps->y = (ga * p1 / (g1) + 0.5 * ro1 * (u1 * u1 + v1 * v1)) * u_L;
        Pu->x = (FL1) * n1 + (FL2) * t1;
        Pu->y = (FL1) * n2 + (FL2) * t2;
    } else if (SR <= 0.0) {
        q = Q_R * u_R;
        Ps->x = ro2 * u_R;
        Ps->y = (ga * p2 / (g1) + 0.5 * ro2 * (u2 * u2 + v2 * v2)) * u_R;
        Pu->x = (FR1) * n1 + (FR2) * t1;
        Pu->y = (FR1) * n2 + (FR2) * t2;
    } else {
        double SM = ((SR - u_R) * ro2 * u_R - (SL - u_L) * ro1 * u_L - p2 + p1) / ((SR - u_R) * ro2 - (SL - u_L) * ro1);
        double pp = p1 + ro1 * (SL - u_L) * (SM - u_L);
        if (SM <= 0.0) {
            double rr = ro2 * (SR - u_R) / (SR - SM);
            double e = p2 / g1 + 0.5 * ro2 * (u2 * u2 + v2 * v2);
            double ee = ((SR - u_R) * e - p2 * u_R + pp * SM) / (SR - SM);
            q = SR * (rr * Q_R / ro2 - Q_R) + Q_R * u_R;
            Ps->x = SR * (rr - ro2) + ro2 * u_R;
            Ps->y = SR * (ee - e) + (ga * p2 / (g1) + 0.5 * ro2 * (u2 * u2 + v2 * v2)) * u_R;
            double F1 = (ro2 * u_R * u_R + p2) + SR * (rr * SM - ro2 * u_R);
            double F2 = (ro2 * u_R * v_R) + SR * (rr * v_R - ro2 * v_R);
            Pu->x = F1 * n1 + F2 * t1;
            Pu->y = F1 * n2 + F2 * t2;
        } else if (SM >= 0.0) {
            double rr = ro1 * (SL - u_L) / (SL - SM);
            double e = p1 / g1 + 0.5 * ro1 * (u1 * u1 + v1 * v1);
            double ee = ((SL - u_L) * e - p1 * u_L + pp * SM) / (SL - SM);
            q = SL * (rr * Q_L / ro1 - Q_L) + Q_L * u_L;
            Ps->x = SL * (rr - ro1) + ro1 * u_L;
            Ps->y = SL * (ee - e) + (ga * p1 / (g1) + 0.5 * ro1 * (u1 * u1 + v1 * v1)) * u_L;
            double F1 = FL1 + SL * (rr * SM - ro1 * u_L);
            double F2 = FL2 + SL * (rr * v_L - ro1 * v_L);
            Pu->x = F1 * n1 + F2 * t1;
            Pu->y = F1 * n2 + F2 * t2;
        } else {
            q = NAN;
            Ps->x = Ps->y = Pu->x = Pu->y = NAN;
        }
    }
    if (PQ) *PQ = q;
    return time;
}

/* ------------------------------------------------------------------------ */
/* exact Riemann solver (kernel.cu:128-765)                                   */
/* ------------------------------------------------------------------------ */
static void lev(const ora_phys* ph, double enI, double pI, double rI, double enII, double pII,
                double rII, double uuu, double* fee)
{
    double cI = sqrt(ph->ga * pI / rI);
    double cII = sqrt(ph->ga * pII / rII);
    double fI = (uuu - pI) / (rI * cI * sqrt(ph->gp * uuu / pI + ph->gm));
    double fII = 2.0 / ph->g1 * cII * (pow((uuu / pII), ph->gm) - 1.0);
    double f1 = fI + fII;
    double f2 = enI - enII;
    *fee = f1 - f2;
}

/* the margin diagnostic: how close one stopping test |res| <= tol came to
   the other outcome, relative to tol (not part of the reference) */
static void ora_margin(ora_stats* st, double res, double tol)
{
    const double m = fabs(fabs(res) - tol) / tol;
    if (m < st->margin) st->margin = m;
}

/* bisection on [pI, pII] for the shock-rarefaction pattern (kernel.cu:682-749) */
static void devtwo(const ora_phys* ph, ora_stats* st, double enI, double pI, double rI,
                   double enII, double pII, double rII, double* p)
{
    const double epsil = ph->eps;
    double kl = pI, kp = pII, kc = 0.0, ksi, ksir, ksit, um;
    int it = 0;
    lev(ph, enI, pI, rI, enII, pII, rII, kl, &ksi);
    lev(ph, enI, pI, rI, enII, pII, rII, kp, &ksir);
    st->bisect_calls++;
    ora_margin(st, ksi, epsil);
    if (fabs(ksi) <= epsil) { *p = kl; return; }
    ora_margin(st, ksir, epsil);
    if (fabs(ksir) <= epsil) { *p = kp; return; }
    for (;;) {
        it++;
        kc = (kl + kp) / 2.0;
        lev(ph, enI, pI, rI, enII, pII, rII, kc, &ksit);
        ora_margin(st, ksit, epsil);
        if (fabs(ksit) <= epsil) break;
        if (it >= ph->max_iter) { st->bisect_cap++; break; }
        if ((ksi * ksit) <= 0.0) { kp = kc; ksir = ksit; }
        else { kl = kc; ksi = ksit; }
    }
    st->bisect_iters += it;
    um = kc;
    *p = um;
}

/* Newton for the two-shock pattern (kernel.cu:635-680); start = acoustic guess */
static void newton(const ora_phys* ph, ora_stats* st, double enI, double pI, double rI,
                   double enII, double pII, double rII, double* p_out)
{
    const double ga = ph->ga, gp = ph->gp, gm = ph->gm;
    double cI = sqrt(ga * pI / rI);
    double cII = sqrt(ga * pII / rII);
    double pn = pI * rII * cII + pII * rI * cI + (enI - enII) * rI * cI * rII * cII;
    pn = pn / (rI * cI + rII * cII);
    double pee = pn, p;
    int kiter = 0;
    for (;;) {
        p = pn;
        kiter++;
        double fI = (p - pI) / (rI * cI * sqrt(gp * p / pI + gm));
        double fIs = (ga + 1.0) * p / pI + (3.0 * ga - 1.0);
        fIs = fIs / (4.0 * ga * rI * cI * pow((gp * p / pI + gm), (3.0 / 2.0)));
        double fII = (p - pII) / (rII * cII * sqrt(gp * p / pII + gm));
        double fIIs = (ga + 1.0) * p / pII + (3.0 * ga - 1.0);
        fIIs = fIIs / (4.0 * ga * rII * cII * pow((gp * p / pII + gm), (3.0 / 2.0)));
        pn = p - (fI + fII - (enI - enII)) / (fIs + fIIs);
        if (!(fabs(pn / pee - p / pee) >= ph->eps)) break;
        if (kiter >= ph->max_iter) { st->newton_cap++; break; }
    }
    st->newton_calls++;
    st->newton_iters += kiter;
    if (kiter > st->newton_max) st->newton_max = kiter;
    *p_out = pn;
}

static double godunov(const ora_phys* ph, ora_stats* st, d2 Ls, d2 Lu, d2 Rs, d2 Ru,
                      double n1, double n2, d2* Ps, d2* Pu, double rad)
{
    const double ga = ph->ga, g1 = ph->g1, g2 = ph->g2, gm = ph->gm;
    const double gg1 = g1, gg2 = g2, gga = ga, krit = ph->krit, eps = 10e-10, eps8 = ph->eps8;
    double w = 0.0;
    double al = n1, be = n2, ge = 0.0;
    double time = 0.0;
    double al2 = -n2, be2 = n1, ge2 = 0.0;
    double al3 = 0.0, be3 = 0.0, ge3 = 1.0;
    double enI = al * Lu.x + be * Lu.y;
    double teI2 = al2 * Lu.x + be2 * Lu.y;
    double teI3 = al3 * Lu.x + be3 * Lu.y;
    double enII = al * Ru.x + be * Ru.y;
    double teII2 = al2 * Ru.x + be2 * Ru.y;
    double teII3 = al3 * Ru.x + be3 * Ru.y;
    double pI = Ls.y, pII = Rs.y, rI = Ls.x, rII = Rs.x;
    int ipiz = 0;
    if (pI > pII) {
        double eno2 = enII, teo22 = teII2, teo23 = teII3, p2 = pII, r2 = rII;
        double eno1 = enI, teo12 = teI2, teo13 = teI3, p1 = pI, r1 = rI;
        enI = -eno2; teI2 = teo22; teI3 = teo23; pI = p2; rI = r2;
        enII = -eno1; teII2 = teo12; teII3 = teo13; pII = p1; rII = r1;
        w = -w;
        ipiz = 1;
    }
    double cI = 0.0, cII = 0.0;
    if (rI != 0.0) cI = sqrt(ga * pI / rI);
    if (rII != 0.0) cII = sqrt(ga * pII / rII);
    double a = sqrt(rI * (g2 * pII + g1 * pI) / 2.0);
    double Uud = (pII - pI) / a;
    double Urz = -2.0 * cII / g1 * (1.0 - pow((pI / pII), gm));
    double Uvk = -2.0 * (cII + cI) / g1;
    double Udf = enI - enII;
    int il = -2, ip = -2;
    if (!(pI == pII && rI == rII && enI == enII)) {
        const double sc = (cI + cII > 0.0) ? cI + cII : 1.0;
        const double pm = fmin(fabs(Udf - Urz), fmin(fabs(Udf - Uud), fabs(Udf - Uvk))) / sc;
        if (pm < st->pmargin) st->pmargin = pm;
    }
    double p = 0.0, r = 0.0, te2 = 0.0, te3 = 0.0, en = 0.0;

    if (Udf < Uvk) { il = -1; ip = -1; }
    else if ((Udf >= Uvk) && (Udf <= Urz)) {
        p = pI * pow(((Udf - Uvk) / (Urz - Uvk)), (1.0 / gm));
        il = 0; ip = 0;
    } else if ((Udf > Urz) && (Udf <= Uud)) {
        devtwo(ph, st, enI, pI, rI, enII, pII, rII, &p);
        il = 1; ip = 0;
    } else if (Udf > Uud) {
        newton(ph, st, enI, pI, rI, enII, pII, rII, &p);
        il = 1; ip = 1;
    }

    if ((il == 1) && (ip == 1)) {            /* two shocks */
        double aI = sqrt(rI * (g2 / 2.0 * p + g1 / 2.0 * pI));
        double aII = sqrt(rII * (g2 / 2.0 * p + g1 / 2.0 * pII));
        double u = (aI * enI + aII * enII + pI - pII) / (aI + aII);
        double dI = enI - aI / rI;
        double dII = enII + aII / rII;
        double UU = fmax(fabs(dI), fabs(dII));
        time = (UU > eps8) ? krit * rad / UU : krit * rad / eps8;
        if (w <= dI) { en = enI; p = pI; r = rI; te2 = teI2; te3 = teI3; }
        else if ((w > dI) && (w <= u)) { en = u; r = rI * aI / (aI - rI * (enI - u)); te2 = teI2; te3 = teI3; }
        else if ((w > u) && (w < dII)) { en = u; r = rII * aII / (aII + rII * (enII - u)); te2 = teII2; te3 = teII3; }
        else if (w >= dII) { en = enII; p = pII; r = rII; te2 = teII2; te3 = teII3; }
    }
    if ((il == 1) && (ip == 0)) {            /* left shock, right rarefaction */
        double aI = sqrt(rI * (g2 / 2.0 * p + g1 / 2.0 * pI));
        double aII;
        if (fabs(p - pII) < eps) aII = rII * cII;
        else aII = gm * rII * cII * (1.0 - p / pII) / (1.0 - pow((p / pII), gm));
        double u = (aI * enI + aII * enII + pI - pII) / (aI + aII);
        double dI = enI - aI / rI;
        double dII = enII + cII;
        double ddII = u + cII - g1 * (enII - u) / 2.0;
        double UU = fmax(fabs(dI), fabs(dII));
        UU = fmax(UU, fabs(ddII));
        time = (UU > eps8) ? krit * rad / UU : krit * rad / eps8;
        if (w <= dI) { en = enI; p = pI; r = rI; te2 = teI2; te3 = teI3; }
        if ((w > dI) && (w <= u)) { en = u; r = rI * aI / (aI - rI * (enI - u)); te2 = teI2; te3 = teI3; }
        if ((w > u) && (w <= ddII)) {
            double ce = cII - g1 / 2.0 * (enII - u);
            en = u; r = ga * p / ce / ce; te2 = teII2; te3 = teII3;
        }
        if ((w > ddII) && (w < dII)) {
            double ce = -g1 / g2 * (enII - w) + 2.0 / g2 * cII;
            en = w - ce; p = pII * pow((ce / cII), (1.0 / gm)); r = ga * p / ce / ce; te2 = teII2; te3 = teII3;
        }
        if (w >= dII) { en = enII; p = pII; r = rII; te2 = teII2; te3 = teII3; }
    }
    if ((il == 0) && (ip == 0)) {            /* two rarefactions */
        double aI, aII;
        if (fabs(p - pI) < eps) aI = rI * cI;
        else aI = gm * rI * cI * (1.0 - p / pI) / (1.0 - pow((p / pI), gm));
        if (fabs(p - pII) < eps) aII = rII * cII;
        else aII = gm * rII * cII * (1.0 - p / pII) / (1.0 - pow((p / pII), gm));
        double u = (aI * enI + aII * enII + pI - pII) / (aI + aII);
        double dI = enI - cI;
        double ddI = u - cI - g1 * (enI - u) / 2.0;
        double dII = enII + cII;
        double ddII = u + cII - g1 * (enII - u) / 2.0;
        double UU = fmax(fabs(dI), fabs(dII));
        UU = fmax(UU, fabs(ddII));
        UU = fmax(UU, fabs(ddI));
        time = (UU > eps8) ? krit * rad / UU : krit * rad / eps8;
        if (w <= dI) { en = enI; p = pI; r = rI; te2 = teI2; te3 = teI3; }
        if ((w > dI) && (w < ddI)) {
            double ce = g1 / g2 * (enI - w) + 2.0 / g2 * cI;
            en = w + ce; p = pI * pow((ce / cI), (1.0 / gm)); r = ga * p / ce / ce; te2 = teI2; te3 = teI3;
        }
        if ((w >= ddI) && (w <= u)) {
            double ce = cI + g1 / 2.0 * (enI - u);
            en = u; r = ga * p / ce / ce; te2 = teI2; te3 = teI3;
        }
        if ((w > u) && (w <= ddII)) {
            double ce = cII - g1 / 2.0 * (enII - u);
            en = u; r = ga * p / ce / ce; te2 = teII2; te3 = teII3;
        }
        if ((w > ddII) && (w < dII)) {
            double ce = -g1 / g2 * (enII - w) + 2.0 / g2 * cII;
            en = w - ce; p = pII * pow((ce / cII), (1.0 / gm)); r = ga * p / ce / ce; te2 = teII2; te3 = teII3;
        }
        if (w >= dII) { en = enII; p = pII; r = rII; te2 = teII2; te3 = teII3; }
    }
    if ((il == -1) && (ip == -1)) {          /* vacuum */
        st->vacuum++;
        double dI = enI - cI;
        double ddI = enI + 2.0 / gg1 * cI;
        double dII = enII + cII;
        double ddII = enII - 2.0 / gg1 * cII;
        double UU = fmax(fabs(dI), fabs(dII));
        UU = fmax(UU, fabs(ddII));
        UU = fmax(UU, fabs(ddI));
        time = (UU > eps8) ? krit * rad / UU : krit * rad / eps8;
        if (w <= dI) { en = enI; p = pI; r = rI; te2 = teI2; te3 = teI3; }
        if ((w > dI) && (w < ddI)) {
            double ce = gg1 / gg2 * (enI - w) + 2.0 / gg2 * cI;
            en = w + ce; p = pI * pow((ce / cI), (1.0 / gm)); r = gga * p / ce / ce; te2 = teI2; te3 = teI3;
        }
        if ((w >= ddI) && (w <= ddII)) { en = w; p = 0.0; r = 0.0; te2 = 0.0; te3 = 0.0; }
        if ((w > ddII) && (w < dII)) {
            double ce = -gg1 / gg2 * (enII - w) + 2.0 / gg2 * cII;
            en = w - ce; p = pII * pow((ce / cII), (1.0 / gm)); r = gga * p / ce / ce; te2 = teII2; te3 = teII3;
        }
        if (w >= dII) { en = enII; p = pII; r = rII; te2 = teII2; te3 = teII3; }
    }
    if (il == -2) { en = NAN; p = NAN; r = NAN; time = NAN; }

    if (ipiz == 1) { en = -en; w = -w; }
    double uo = al * en + al2 * te2 + al3 * te3;
    double vo = be * en + be2 * te2 + be3 * te3;
    double wo = ge * en + ge2 * te2 + ge3 * te3;
    double eo = p / g1 + 0.5 * r * (uo * uo + vo * vo + wo * wo);
    en = al * uo + be * vo + ge * wo;
    Ps->x = (r * (en - w));
    Pu->x = (r * (en - w) * uo + al * p);
    Pu->y = (r * (en - w) * vo + be * p);
    Ps->y = ((en - w) * eo + en * p);
    return time;
}

/* ------------------------------------------------------------------------ */
/* exported face functions (for the pinning tests)                           */
/* in: sL=(rho,p) uL=(vz,vr) sR uR; out[4] = (mass, mom_z, mom_r, energy)    */
/* ------------------------------------------------------------------------ */
/* ------------------------------------------------------------------------ */
/* HLLC_Aleksashov (kernel.cu:767-1079): an MHD HLLC solver that the        */
/* reference calls with zero magnetic field.  With B = 0 its frame is the   */
/* normal n, the third axis and t = (-n_y, n_x) (the branch d <= eps of its */
/* frame construction; d = 1), the fast speed is sqrt(c c), the tangential  */
/* star velocities are the side's own, and the magnetic terms add zeros,    */
/* which are left out here (adding +0 to a nonzero sum changes nothing).    */
/* ------------------------------------------------------------------------ */
static double hllc_a(const ora_phys* ph, d2 Ls, d2 Lu, d2 Rs, d2 Ru, double n1, double n2,
                     d2* Ps, d2* Pu, double rad)
{
    const double ga = ph->ga, g1 = ph->g1, wv = 0.0;
    const double r1 = Ls.x, p1 = Ls.y, u1 = Lu.x, v1 = Lu.y;
    const double r2 = Rs.x, p2 = Rs.y, u2 = Ru.x, v2 = Ru.y;
    /* frame: columns a0 = n, a1 = (0, 0, 1), a2 = (-n_y, n_x, 0) */
    const double a02 = (0.0 * 0.0 - 1.0 * n2), a12 = (1.0 * n1 - 0.0 * 0.0);
    const double vL0 = n1 * u1 + n2 * v1, vR0 = n1 * u2 + n2 * v2;
    const double vL2 = a02 * u1 + a12 * v1, vR2 = a02 * u2 + a12 * v2;
    const double cL = sqrt(ga * p1 / r1), cR = sqrt(ga * p2 / r2);
    const double cfL = sqrt(cL * cL), cfR = sqrt(cR * cR);
    const double SL = fmin(vL0 - cfL, vR0 - cfR);
    const double SR = fmax(vL0 + cfL, vR0 + cfR);
    const double suR = SR - vR0, suL = SL - vL0;
    const double SM = (suR * r2 * vR0 - p2 + p1 - suL * r1 * vL0) / (suR * r2 - suL * r1);
    const double UU = fmax(fabs(SL), fabs(SR));
    const double time = ph->krit * rad / UU;
    const double upt1 = (u1 * u1 + v1 * v1) / 2.0, upt2 = (u2 * u2 + v2 * v2) / 2.0;
    const double e1 = p1 / g1 + r1 * upt1, e2 = p2 / g1 + r2 * upt2;
    /* side fluxes and conserved states: mass, normal / tangential momentum, energy */
    const double FL[4] = {r1 * vL0, r1 * vL0 * vL0 + p1, r1 * vL0 * vL2, (e1 + p1) * vL0};
    const double FR[4] = {r2 * vR0, r2 * vR0 * vR0 + p2, r2 * vR0 * vR2, (e2 + p2) * vR0};
    const double UL[4] = {r1, r1 * vL0, r1 * vL2, e1};
    const double UR[4] = {r2, r2 * vR0, r2 * vR2, e2};
    const double suRm = suR / (SR - SM), suLm = suL / (SL - SM);
    const double rzR = r2 * suRm, rzL = r1 * suLm;
    const double ptzR = p2 + r2 * suR * (SM - vR0);
    const double ptzL = p1 + r1 * suL * (SM - vL0);
    const double ptz = (ptzR + ptzL) / 2.0;
    const double ezR = e2 * suRm + (ptz * SM - p2 * vR0) / (SR - SM);
    const double ezL = e1 * suLm + (ptz * SM - p1 * vL0) / (SL - SM);
    const double UZL[4] = {rzL, SM * rzL, vL2 * rzL, ezL};
    const double UZR[4] = {rzR, SM * rzR, vR2 * rzR, ezR};
    double q[4];
    if (SL > wv) {
        for (int k = 0; k < 4; k++) q[k] = FL[k] - wv * UL[k];
    } else if ((SL <= wv) && (SM >= wv)) {
        for (int k = 0; k < 4; k++) q[k] = FL[k] + SL * (UZL[k] - UL[k]) - wv * UZL[k];
    } else if ((SM <= wv) && (SR >= wv)) {
        for (int k = 0; k < 4; k++) q[k] = FR[k] + SR * (UZR[k] - UR[k]) - wv * UZR[k];
    } else if (SR < wv) {
        for (int k = 0; k < 4; k++) q[k] = FR[k] - wv * UR[k];
    } else {
        for (int k = 0; k < 4; k++) q[k] = NAN;
    }
    Ps->x = q[0];
    Ps->y = q[3];
    Pu->x = n1 * q[1] + a02 * q[2];
    Pu->y = n2 * q[1] + a12 * q[2];
    return time;
}

static void pack_out(d2 Ps, d2 Pu, double* out)
{
    out[0] = Ps.x; out[1] = Pu.x; out[2] = Pu.y; out[3] = Ps.y;
}

double ora_face(int flux, double gamma, double krit, double tol, int max_iter,
                const double* sL, const double* uL, const double* sR, const double* uR,
                double n1, double n2, double rad, double* out, int64_t* counters)
{
    ora_phys ph;
    ora_stats st;
    memset(&st, 0, sizeof st);
    ora_phys_init(&ph, gamma, krit, tol, max_iter);
    d2 Ls = {sL[0], sL[1]}, Lu = {uL[0], uL[1]}, Rs = {sR[0], sR[1]}, Ru = {uR[0], uR[1]};
    d2 Ps = {0, 0}, Pu = {0, 0};
    double t;
    if (flux == AST_FLUX_HLL) t = hll(&ph, Ls, Lu, Rs, Ru, n1, n2, &Ps, &Pu, rad);
    else if (flux == AST_FLUX_HLLC) t = hllc(&ph, Ls, Lu, Rs, Ru, n1, n2, &Ps, &Pu, rad, 0);
    else if (flux == AST_FLUX_HLLC_A) t = hllc_a(&ph, Ls, Lu, Rs, Ru, n1, n2, &Ps, &Pu, rad);
    else if (flux == AST_FLUX_HLLCQ) t = hllcq(&ph, Ls, Lu, Rs, Ru, 0.0, 0.0, n1, n2, &Ps, &Pu, NULL, rad);
    else t = godunov(&ph, &st, Ls, Lu, Rs, Ru, n1, n2, &Ps, &Pu, rad);
    pack_out(Ps, Pu, out);
    if (counters) {
        counters[0] = st.newton_calls; counters[1] = st.newton_iters; counters[2] = st.newton_cap;
        counters[3] = st.bisect_calls; counters[4] = st.bisect_iters; counters[5] = st.bisect_cap;
        counters[6] = st.vacuum;
    }
    return t;
}

/* One face of the passive-scalar solvers (flux AST_FLUX_HLLC: the Q channel
   of HLLC_2d_Korolkov_b_s; AST_FLUX_HLLCQ: HLLCQ_Korolkov_2D): out[0..3] as
   ora_face, out[4] the scalar's flux; returns the face dt. */
double ora_face_q(int flux, double gamma, double krit, const double* sL, const double* uL, const double* sR,
                  const double* uR, double QL, double QR, double n1, double n2, double rad, double* out)
{
    ora_phys ph;
    ora_phys_init(&ph, gamma, krit, 10e-10, 200);
    d2 Ls = {sL[0], sL[1]}, Lu = {uL[0], uL[1]}, Rs = {sR[0], sR[1]}, Ru = {uR[0], uR[1]};
    d2 Ps = {0, 0}, Pu = {0, 0};
    double PQ = 0.0, t;
    if (flux == AST_FLUX_HLLCQ) t = hllcq(&ph, Ls, Lu, Rs, Ru, QL, QR, n1, n2, &Ps, &Pu, &PQ, rad);
    else t = hllc_q(&ph, Ls, Lu, Rs, Ru, QL, QR, n1, n2, &Ps, &Pu, &PQ, rad, 0);
    pack_out(Ps, Pu, out);
    out[4] = PQ;
    return t;
}

/* ------------------------------------------------------------------------ */
/* grid and ghost cells                                                      */
/* ------------------------------------------------------------------------ */
typedef struct ora_grid {
    int N, M;
    double x_min, dx, y_min, dy;
} ora_grid;

static void ora_grid_init(ora_grid* g, const ast_config* c)
{
    g->N = c->N;
    g->M = c->M;
    g->x_min = c->x_min;
    g->dx = (c->x_max - c->x_min) / (c->N - 1);        /* Header.h:15 */
    g->dy = (c->y_max) / (c->M);                       /* Header.h:16 */
    g->y_min = (c->y_max / (2.0 * c->M));              /* Header.h:14 */
}

/* state at (n, m), with the ghost rules of the side that (n, m) lies beyond */
static void ora_get(const ora_grid* g, const ast_config* c, const d2* s, const d2* u,
                    int n, int m, d2* so, d2* uo)
{
    const int N = g->N, M = g->M;
    if (n >= 0 && n < N && m >= 0 && m < M) {
        *so = s[m * N + n]; *uo = u[m * N + n];
        return;
    }
    int side, j, b0, mir, low;
    if (n < 0)       { side = AST_Z_LO; j = -1 - n; b0 = m * N + 0;       mir = m * N + j;           low = 1; }
    else if (n >= N) { side = AST_Z_HI; j = n - N;  b0 = m * N + N - 1;   mir = m * N + (N - 1 - j); low = 0; }
    else if (m < 0)  { side = AST_R_LO; j = -1 - m; b0 = 0 * N + n;       mir = j * N + n;           low = 1; }
    else             { side = AST_R_HI; j = m - M;  b0 = (M - 1) * N + n; mir = (M - 1 - j) * N + n; low = 0; }
    const ast_bc* bc = &c->bc[side];
    const int zside = (side == AST_Z_LO || side == AST_Z_HI);
    switch (bc->kind) {
    case AST_BC_REFLECT:
        *so = s[mir]; *uo = u[mir];
        if (zside) uo->x = -uo->x; else uo->y = -uo->y;
        break;
    case AST_BC_FIXED:
        so->x = bc->rho; so->y = bc->p; uo->x = bc->vz; uo->y = bc->vr;
        break;
    case AST_BC_SUCTION: {
        *so = s[b0]; *uo = u[b0];
        double* vn = zside ? &uo->x : &uo->y;
        double lim = zside ? bc->vz : bc->vr;
        if (low) { if (*vn > lim) *vn = lim; }
        else     { if (*vn < lim) *vn = lim; }
        break;
    }
    case AST_BC_NONREFLECT: {
        /* kernel.cu:1979-1985 (commented there), along the outward normal */
        *so = s[b0]; *uo = u[b0];
        double* vn = zside ? &uo->x : &uo->y;
        double w = low ? -*vn : *vn;
        double ggg = c->gamma;
        double cc = sqrt(ggg * so->y / so->x);
        double cg = (ggg - 1.0) / (ggg + 1.0) * (w + 2.0 / (ggg - 1.0) * cc);
        so->x = so->x * pow(cg / cc, 2.0 / (ggg - 1.0));
        so->y = so->x * cg * cg / ggg;
        *vn = low ? -cg : cg;
        break;
    }
    default: /* OUTFLOW */
        *so = s[b0]; *uo = u[b0];
        break;
    }
}

#ifdef ORA_WITH_REF
/* Built into oracle/_ref/libastref.so: every face is evaluated by the
   reference's own function (HLL kernel.cu:1399, HLLC_2d_Korolkov
   Gas_Dinamic.cu:1814, Godunov_Solver_Alexashov kernel.cu:128,
   HLLCQ_Korolkov_2D Gas_Dinamic.cu:249), compiled for the host by
   oracle/ref_driver.cpp; gamma and CFL come from ref_set_params. */
double ref_face(int which, const double* sL, const double* uL, const double* sR, const double* uR,
                double n1, double n2, double rad, double* out);
double ref_face_q(int which, const double* sL, const double* uL, const double* sR, const double* uR, double QL,
                  double QR, double n1, double n2, double rad, double* out);
#define REF_WHICH(flux) ((flux) == AST_FLUX_HLLCQ ? 5 : (flux))
#endif

static double ora_flux(int flux, const ora_phys* ph, ora_stats* st, d2 Ls, d2 Lu, d2 Rs, d2 Ru,
                       double n1, double n2, d2* Ps, d2* Pu, double rad)
{
#ifdef ORA_WITH_REF
    (void)ph; (void)st;
    double sl[2] = {Ls.x, Ls.y}, ul[2] = {Lu.x, Lu.y}, sr[2] = {Rs.x, Rs.y}, ur[2] = {Ru.x, Ru.y}, out[4];
    double t = ref_face(REF_WHICH(flux), sl, ul, sr, ur, n1, n2, rad, out);
    Ps->x = out[0]; Pu->x = out[1]; Pu->y = out[2]; Ps->y = out[3];
    return t;
#endif
    if (flux == AST_FLUX_HLLC) return hllc(ph, Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad, 0);
    if (flux == AST_FLUX_HLLCQ) return hllcq(ph, Ls, Lu, Rs, Ru, 0.0, 0.0, n1, n2, Ps, Pu, NULL, rad);
    if (flux == AST_FLUX_HLLC_A) return hllc_a(ph, Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad);
    if (flux == AST_FLUX_GODUNOV) return godunov(ph, st, Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad);
    return hll(ph, Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad);
}

/* a face of the passive-scalar step: the gas flux as ora_flux gives it and
   the scalar's flux *PQ (flux HLLC or HLLCQ) */
static double ora_flux_q(int flux, const ora_phys* ph, ora_stats* st, d2 Ls, d2 Lu, d2 Rs, d2 Ru, double QL,
                         double QR, double n1, double n2, d2* Ps, d2* Pu, double* PQ, double rad)
{
    (void)st;
#ifdef ORA_WITH_REF
    (void)ph;
    double sl[2] = {Ls.x, Ls.y}, ul[2] = {Lu.x, Lu.y}, sr[2] = {Rs.x, Rs.y}, ur[2] = {Ru.x, Ru.y}, out[5];
    double t = ref_face_q(REF_WHICH(flux), sl, ul, sr, ur, QL, QR, n1, n2, rad, out);
    Ps->x = out[0]; Pu->x = out[1]; Pu->y = out[2]; Ps->y = out[3]; *PQ = out[4];
    return t;
#endif
    if (flux == AST_FLUX_HLLCQ) return hllcq(ph, Ls, Lu, Rs, Ru, QL, QR, n1, n2, Ps, Pu, PQ, rad);
    return hllc_q(ph, Ls, Lu, Rs, Ru, QL, QR, n1, n2, Ps, Pu, PQ, rad, 0);
}

/* neighbour-side face value with the positivity rule (kernel.cu:2801-2850) */
static d2 nb_s(double c0, double h, double hh, d2 s1, d2 sn, d2 sn2, int grad_p)
{
    /* c0: own centre, h: +-d (toward neighbour), hh: +-d/2 (the face) */
    d2 r;
    r.x = ora_linear(c0, s1.x, c0 + h, sn.x, c0 + 2.0 * h, sn2.x, c0 + hh);
    if (r.x <= 0) r.x = sn.x;
    r.y = ora_linear(c0, s1.y, c0 + h, sn.y, c0 + 2.0 * h, sn2.y, c0 + hh);
    if ((r.y <= 0) || (!grad_p)) r.y = sn.y;
    return r;
}

static d2 nb_u(double c0, double h, double hh, d2 u1, d2 un, d2 un2)
{
    d2 r;
    r.x = ora_linear(c0, u1.x, c0 + h, un.x, c0 + 2.0 * h, un2.x, c0 + hh);
    r.y = ora_linear(c0, u1.y, c0 + h, un.y, c0 + 2.0 * h, un2.y, c0 + hh);
    return r;
}

static int in_region(const ast_config* c, double xf)
{
    return !c->region_select || (xf > c->region_lo && xf < c->region_hi);
}

/* The neutral-coupling source nn2 (K x, y, z triples, the reference's
   double3 layout) the steps use, or NULL for none.  The array is read, not
   copied: it must outlive the steps. */
static const double* g_nn2 = NULL;

void ora_set_neutral(const double* nn2) { g_nn2 = nn2; }

/* Per-cell margin diagnostic (not part of the reference): when set, every
   step writes, for each cell k, the smallest | |res| - tol | / tol over the
   bisection stopping tests of its four faces (devtwo, kernel.cu:682-749),
   or a large value when none ran.  A cell whose margin is small can take one
   bisection iterate more or less under rounding of its inputs. */
static double* g_margin = NULL;
static double* g_pmargin = NULL;

/* per_cell: the bisection margins; pattern (may be NULL): per cell the
   smallest distance of Udf to a wave-pattern threshold of its faces
   (Uvk, Urz, Uud of kernel.cu:186-231) relative to cI + cII, over the faces
   with unequal states (a cell whose faces sit on a threshold can change
   pattern under rounding of its inputs) */
void ora_set_margin(double* per_cell, double* pattern) { g_margin = per_cell; g_pmargin = pattern; }

/* The passive scalar the steps carry (ora_set_scalar): Q of the old state,
   Q of the new, and its value in FIXED ghost cells; NULL for none.  Its
   ghost rules are the state's (mirror, copy of the boundary cell, fixed
   value); its face values are reconstructed with the density's rule. */
static const double* g_q = NULL;
static double* g_q2 = NULL;
static double g_q_fixed = 0.0;

void ora_set_scalar(const double* q, double* q2, double q_fixed)
{
    g_q = q;
    g_q2 = q2;
    g_q_fixed = q_fixed;
}

static double ora_get_q(const ora_grid* g, const ast_config* c, int n, int m)
{
    const int N = g->N, M = g->M;
    if (n >= 0 && n < N && m >= 0 && m < M) return g_q[m * N + n];
    int side, j, b0, mir;
    if (n < 0)       { side = AST_Z_LO; j = -1 - n; b0 = m * N + 0;       mir = m * N + j; }
    else if (n >= N) { side = AST_Z_HI; j = n - N;  b0 = m * N + N - 1;   mir = m * N + (N - 1 - j); }
    else if (m < 0)  { side = AST_R_LO; j = -1 - m; b0 = 0 * N + n;       mir = j * N + n; }
    else             { side = AST_R_HI; j = m - M;  b0 = (M - 1) * N + n; mir = (M - 1 - j) * N + n; }
    if (c->bc[side].kind == AST_BC_REFLECT) return g_q[mir];
    if (c->bc[side].kind == AST_BC_FIXED) return g_q_fixed;
    return g_q[b0];
}

/* neighbour-side face value of the scalar (the density's rule) */
static double nb_q(double c0, double h, double hh, double q1, double qn, double qn2)
{
    double r = ora_linear(c0, q1, c0 + h, qn, c0 + 2.0 * h, qn2, c0 + hh);
    return (r <= 0) ? qn : r;
}

/* a high-order face: with the scalar, its flux *PQ beside the gas flux */
static double face_call(int flux, const ora_phys* ph, ora_stats* st, d2 Ls, d2 Lu, d2 Rs, d2 Ru, double ql,
                        double qr, double n1, double n2, d2* Ps, d2* Pu, double* PQ, double rad)
{
    if (g_q) return ora_flux_q(flux, ph, st, Ls, Lu, Rs, Ru, ql, qr, n1, n2, Ps, Pu, PQ, rad);
    *PQ = 0.0;
    return ora_flux(flux, ph, st, Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad);
}

/* One cell of one step.  Returns the cell's tmin; a cell held fixed returns
   1e7, the reset value of T, because the reference's fixed cells never
   touch T (kernel.cu:2318-2324). */
static double ora_cell(const ora_grid* g, const ast_config* c, const ora_phys* ph, ora_stats* st,
                       const d2* s, const d2* u, d2* s2, d2* u2, int n, int m, double T_do)
{
    const int N = g->N;
    const int index = m * N + n;
    const double dx = g->dx, dy = g->dy;
    const double y = g->y_min + m * dy;
    const double x = g->x_min + n * dx;
    const double ggg = ph->ga;
    double tmin = c->dt_cap;
    d2 s_1 = s[index], u_1 = u[index];
    st->margin = 1e300;
    st->pmargin = 1e300;

    if (c->fixed_region) {
        double xz = x - c->fixed_zc;
        double dist2 = (xz * xz) / (c->fixed_az * c->fixed_az) + (y * y) / (c->fixed_ar * c->fixed_ar);
        if (dist2 < 1.0) {
            s2[index] = s_1; u2[index] = u_1;
            if (g_q) g_q2[index] = g_q[index];
            return 10000000;
        }
    }
    /* the scalar's stencil and its cell-side face values */
    double q_1 = 0, q_2 = 0, q_3 = 0, q_4 = 0, q_5 = 0, q21 = 0, q31 = 0, q41 = 0, q51 = 0;
    double PQ12 = 0, PQ13 = 0, PQ14 = 0, PQ15 = 0;
    if (g_q) {
        q_1 = g_q[index];
        q_2 = ora_get_q(g, c, n + 1, m); q_3 = ora_get_q(g, c, n, m - 1);
        q_4 = ora_get_q(g, c, n - 1, m); q_5 = ora_get_q(g, c, n, m + 1);
        q21 = ora_get_q(g, c, n + 2, m); q31 = ora_get_q(g, c, n, m - 2);
        q41 = ora_get_q(g, c, n - 2, m); q51 = ora_get_q(g, c, n, m + 2);
    }
    double q12 = q_1, q13 = q_1, q14 = q_1, q15 = q_1;

    d2 s_2, s_3, s_4, s_5, u_2, u_3, u_4, u_5;
    ora_get(g, c, s, u, n + 1, m, &s_2, &u_2);
    ora_get(g, c, s, u, n, m - 1, &s_3, &u_3);
    ora_get(g, c, s, u, n - 1, m, &s_4, &u_4);
    ora_get(g, c, s, u, n, m + 1, &s_5, &u_5);

    d2 Ps12 = {0, 0}, Pu12 = {0, 0}, Ps13 = {0, 0}, Pu13 = {0, 0};
    d2 Ps14 = {0, 0}, Pu14 = {0, 0}, Ps15 = {0, 0}, Pu15 = {0, 0};
    const int recon = (c->recon == AST_RECON_MINMOD);
    const int gp = c->grad_p;
    d2 s12 = s_1, s13 = s_1, s14 = s_1, s15 = s_1, u12 = u_1, u13 = u_1, u14 = u_1, u15 = u_1;
    d2 s21 = {0, 0}, s31 = {0, 0}, s41 = {0, 0}, s51 = {0, 0};
    d2 u21 = {0, 0}, u31 = {0, 0}, u41 = {0, 0}, u51 = {0, 0};
    if (recon) {
        double A, B;
        ora_get(g, c, s, u, n + 2, m, &s21, &u21);
        ora_get(g, c, s, u, n - 2, m, &s41, &u41);
        ora_get(g, c, s, u, n, m + 2, &s51, &u51);
        ora_get(g, c, s, u, n, m - 2, &s31, &u31);
        /* cell-side face values (kernel.cu:2704-2796) */
        ora_linear2(x - dx, s_4.x, x, s_1.x, x + dx, s_2.x, x - dx / 2.0, x + dx / 2.0, &A, &B);
        s12.x = (B <= 0) ? s_1.x : B;
        s14.x = (A <= 0) ? s_1.x : A;
        ora_linear2(x - dx, s_4.y, x, s_1.y, x + dx, s_2.y, x - dx / 2.0, x + dx / 2.0, &A, &B);
        s12.y = ((B <= 0) || !gp) ? s_1.y : B;
        s14.y = ((A <= 0) || !gp) ? s_1.y : A;
        ora_linear2(x - dx, u_4.x, x, u_1.x, x + dx, u_2.x, x - dx / 2.0, x + dx / 2.0, &A, &B);
        u12.x = B; u14.x = A;
        ora_linear2(x - dx, u_4.y, x, u_1.y, x + dx, u_2.y, x - dx / 2.0, x + dx / 2.0, &A, &B);
        u12.y = B; u14.y = A;
        ora_linear2(y - dy, s_3.x, y, s_1.x, y + dy, s_5.x, y - dy / 2.0, y + dy / 2.0, &A, &B);
        s15.x = (B <= 0) ? s_1.x : B;
        s13.x = (A <= 0) ? s_1.x : A;
        ora_linear2(y - dy, s_3.y, y, s_1.y, y + dy, s_5.y, y - dy / 2.0, y + dy / 2.0, &A, &B);
        s15.y = ((B <= 0) || !gp) ? s_1.y : B;
        s13.y = ((A <= 0) || !gp) ? s_1.y : A;
        ora_linear2(y - dy, u_3.x, y, u_1.x, y + dy, u_5.x, y - dy / 2.0, y + dy / 2.0, &A, &B);
        u15.x = B; u13.x = A;
        ora_linear2(y - dy, u_3.y, y, u_1.y, y + dy, u_5.y, y - dy / 2.0, y + dy / 2.0, &A, &B);
        u15.y = B; u13.y = A;
        if (g_q) {
            ora_linear2(x - dx, q_4, x, q_1, x + dx, q_2, x - dx / 2.0, x + dx / 2.0, &A, &B);
            q12 = (B <= 0) ? q_1 : B;
            q14 = (A <= 0) ? q_1 : A;
            ora_linear2(y - dy, q_3, y, q_1, y + dy, q_5, y - dy / 2.0, y + dy / 2.0, &A, &B);
            q15 = (B <= 0) ? q_1 : B;
            q13 = (A <= 0) ? q_1 : A;
        }
    }

    double t;
    /* face 12: +z, rad dx (kernel.cu:2799-2813) */
    if (in_region(c, x + dx / 2.0)) {
        if (recon) {
            d2 rs = nb_s(x, dx, dx / 2.0, s_1, s_2, s21, gp), ru = nb_u(x, dx, dx / 2.0, u_1, u_2, u21);
            double rq = g_q ? nb_q(x, dx, dx / 2.0, q_1, q_2, q21) : 0.0;
            t = face_call(c->flux, ph, st, s12, u12, rs, ru, q12, rq, 1, 0, &Ps12, &Pu12, &PQ12, dx);
        } else {
            t = face_call(c->flux, ph, st, s_1, u_1, s_2, u_2, q_1, q_2, 1, 0, &Ps12, &Pu12, &PQ12, dx);
        }
    } else {
        t = ora_flux(AST_FLUX_HLL, ph, st, s_1, u_1, s_2, u_2, 1, 0, &Ps12, &Pu12, dx);
    }
    tmin = fmin(tmin, t);
    /* faces 13 (-r) and 15 (+r), rad dy (kernel.cu:2816-2840) */
    if (in_region(c, x)) {
        if (recon) {
            d2 rs = nb_s(y, -dy, -dy / 2.0, s_1, s_3, s31, gp), ru = nb_u(y, -dy, -dy / 2.0, u_1, u_3, u31);
            double rq = g_q ? nb_q(y, -dy, -dy / 2.0, q_1, q_3, q31) : 0.0;
            t = face_call(c->flux, ph, st, s13, u13, rs, ru, q13, rq, 0, -1, &Ps13, &Pu13, &PQ13, dy);
            tmin = fmin(tmin, t);
            rs = nb_s(y, dy, dy / 2.0, s_1, s_5, s51, gp); ru = nb_u(y, dy, dy / 2.0, u_1, u_5, u51);
            rq = g_q ? nb_q(y, dy, dy / 2.0, q_1, q_5, q51) : 0.0;
            t = face_call(c->flux, ph, st, s15, u15, rs, ru, q15, rq, 0, 1, &Ps15, &Pu15, &PQ15, dy);
            tmin = fmin(tmin, t);
        } else {
            t = face_call(c->flux, ph, st, s_1, u_1, s_3, u_3, q_1, q_3, 0, -1, &Ps13, &Pu13, &PQ13, dy);
            tmin = fmin(tmin, t);
            t = face_call(c->flux, ph, st, s_1, u_1, s_5, u_5, q_1, q_5, 0, 1, &Ps15, &Pu15, &PQ15, dy);
            tmin = fmin(tmin, t);
        }
    } else {
        t = ora_flux(AST_FLUX_HLL, ph, st, s_1, u_1, s_3, u_3, 0, -1, &Ps13, &Pu13, dy);
        tmin = fmin(tmin, t);
        t = ora_flux(AST_FLUX_HLL, ph, st, s_1, u_1, s_5, u_5, 0, 1, &Ps15, &Pu15, dy);
        tmin = fmin(tmin, t);
    }
    /* face 14: -z, rad dx (kernel.cu:2843-2857) */
    if (in_region(c, x - dx / 2.0)) {
        if (recon) {
            d2 rs = nb_s(x, -dx, -dx / 2.0, s_1, s_4, s41, gp), ru = nb_u(x, -dx, -dx / 2.0, u_1, u_4, u41);
            double rq = g_q ? nb_q(x, -dx, -dx / 2.0, q_1, q_4, q41) : 0.0;
            t = face_call(c->flux, ph, st, s14, u14, rs, ru, q14, rq, -1, 0, &Ps14, &Pu14, &PQ14, dx);
        } else {
            t = face_call(c->flux, ph, st, s_1, u_1, s_4, u_4, q_1, q_4, -1, 0, &Ps14, &Pu14, &PQ14, dx);
        }
    } else {
        t = ora_flux(AST_FLUX_HLL, ph, st, s_1, u_1, s_4, u_4, -1, 0, &Ps14, &Pu14, dx);
    }
    tmin = fmin(tmin, t);

    /* neutral-coupling momentum source of add_MK (kernel.cu:2495-2496):
       T_do * (rho * n_H / Kn) * nn2[index].(x, y), with the reference's
       expression order; its energy term multiplies nn3 by 0 */
    double NSx = 0.0, NSy = 0.0;
    if (g_nn2 && c->neutral_kn != 0.0) {
        NSx = T_do * (s_1.x * c->neutral_nh / c->neutral_kn) * g_nn2[3 * (size_t)index];
        NSy = T_do * (s_1.x * c->neutral_nh / c->neutral_kn) * g_nn2[3 * (size_t)index + 1];
    }

    /* body force (kernel.cu:3034-3056) */
    double Q2x = 0.0, Q2 = 0.0, Q3;
    if (c->body_force && x > c->body_lo && x < c->body_hi)
        Q2 = (y >= c->body_rsplit) ? -c->body_amp * s_1.x : c->body_amp * s_1.x;
    Q3 = Q2x * u_1.x + Q2 * u_1.y;

    d2 PS, PU, rs2, ru2;
    const double dV = dx * dy;
    if (c->geom == AST_GEOM_AXISYM) {
        /* add_MK update with its cylindrical source (kernel.cu:2480-2509) */
        PS.x = (Ps12.x + Ps14.x) * dy + (Ps13.x + Ps15.x) * dx;
        PS.y = (Ps12.y + Ps14.y) * dy + (Ps13.y + Ps15.y) * dx;
        PU.x = (Pu12.x + Pu14.x) * dy + (Pu13.x + Pu15.x) * dx;
        PU.y = (Pu12.y + Pu14.y) * dy + (Pu13.y + Pu15.y) * dx;
        rs2.x = s_1.x - (T_do / dV) * PS.x - (T_do / y) * s_1.x * u_1.y;
        if (rs2.x <= 0) { st->rho_floor++; rs2.x = s_1.x; }
        ru2.x = (s_1.x * u_1.x - (T_do / dV) * PU.x - (T_do / y) * s_1.x * u_1.y * u_1.x + T_do * Q2x + NSx) / rs2.x;
        ru2.y = (s_1.x * u_1.y - (T_do / dV) * PU.y - (T_do / y) * s_1.x * u_1.y * u_1.y + T_do * Q2 + NSy) / rs2.x;
        rs2.y = (((s_1.y / (ggg - 1.0) + s_1.x * (u_1.x * u_1.x + u_1.y * u_1.y) * 0.5) - (T_do / dV) * PS.y -
                  (T_do / y) * u_1.y * (ggg * s_1.y / (ggg - 1.0) + s_1.x * (u_1.x * u_1.x + u_1.y * u_1.y) * 0.5) +
                  T_do * Q3) -
                 0.5 * rs2.x * (ru2.x * ru2.x + ru2.y * ru2.y)) * (ggg - 1.0);
    } else {
        /* Kernel_TVD update (kernel.cu:3027-3073) */
        PS.x = Ps12.x * dy + Ps13.x * dx + Ps14.x * dy + Ps15.x * dx;
        PS.y = Ps12.y * dy + Ps13.y * dx + Ps14.y * dy + Ps15.y * dx;
        PU.x = Pu12.x * dy + Pu13.x * dx + Pu14.x * dy + Pu15.x * dx;
        PU.y = Pu12.y * dy + Pu13.y * dx + Pu14.y * dy + Pu15.y * dx;
        rs2.x = s_1.x - (T_do / dV) * PS.x;
        if (rs2.x <= 0.0) { st->rho_floor++; rs2.x = s_1.x; }
        ru2.x = (s_1.x * u_1.x - (T_do / dV) * PU.x + T_do * Q2x + NSx) / rs2.x;
        ru2.y = (s_1.x * u_1.y - (T_do / dV) * PU.y + T_do * Q2 + NSy) / rs2.x;
        rs2.y = (((s_1.y / (ggg - 1) + s_1.x * (u_1.x * u_1.x + u_1.y * u_1.y) * 0.5) - (T_do / dV) * PS.y + T_do * Q3) -
                 0.5 * rs2.x * (ru2.x * ru2.x + ru2.y * ru2.y)) * (ggg - 1);
    }
    if (rs2.y <= 0.0) { st->p_floor++; rs2.y = c->p_floor; }
    s2[index] = rs2;
    u2[index] = ru2;
    if (g_q) {
        /* the scalar in the density's update form */
        double PQS;
        if (c->geom == AST_GEOM_AXISYM) {
            PQS = (PQ12 + PQ14) * dy + (PQ13 + PQ15) * dx;
            g_q2[index] = q_1 - (T_do / dV) * PQS - (T_do / y) * q_1 * u_1.y;
        } else {
            PQS = PQ12 * dy + PQ13 * dx + PQ14 * dy + PQ15 * dx;
            g_q2[index] = q_1 - (T_do / dV) * PQS;
        }
    }
    return tmin;
}

static void stats_add(ora_stats* a, const ora_stats* b)
{
    a->rho_floor += b->rho_floor; a->p_floor += b->p_floor;
    a->newton_calls += b->newton_calls; a->newton_iters += b->newton_iters; a->newton_cap += b->newton_cap;
    a->bisect_calls += b->bisect_calls; a->bisect_iters += b->bisect_iters; a->bisect_cap += b->bisect_cap;
    a->vacuum += b->vacuum;
    if (b->newton_max > a->newton_max) a->newton_max = b->newton_max;
}

/*
 * One step: (s, u) -> (s2, u2) with the lagged T_do.  Returns the new dt,
 * min(1e7, min over active cells of tmin) exactly as Kernel_TVD + funk_time
 * produce it (kernel.cu:3013-3017, 1527-1529).  s, u, s2, u2 hold K pairs.
 * counters (optional, 10 int64): rho_floor, p_floor, newton_calls,
 * newton_iters, newton_cap, bisect_calls, bisect_iters, bisect_cap, vacuum,
 * newton_max (accumulated).
 */
double ora_step(const ast_config* c, const double* s, const double* u, double* s2, double* u2,
                double T_do, int nthreads, int64_t* counters)
{
    ora_grid g;
    ora_phys ph;
    ora_grid_init(&g, c);
    ora_phys_init(&ph, c->gamma, c->cfl, c->riemann_tol, c->riemann_max_iter);
    ora_stats total;
    memset(&total, 0, sizeof total);
    double T = 10000000;
    const d2* S = (const d2*)s;
    const d2* U = (const d2*)u;
    d2* S2 = (d2*)s2;
    d2* U2 = (d2*)u2;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        ora_stats st;
        memset(&st, 0, sizeof st);
        double Tl = 10000000;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int m = 0; m < g.M; m++) {
            for (int n = 0; n < g.N; n++) {
                double tm = ora_cell(&g, c, &ph, &st, S, U, S2, U2, n, m, T_do);
                if (Tl > tm) Tl = tm;
                if (g_margin) g_margin[(size_t)m * g.N + n] = st.margin;
                if (g_pmargin) g_pmargin[(size_t)m * g.N + n] = st.pmargin;
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            if (T > Tl) T = Tl;
            stats_add(&total, &st);
        }
    }
    if (counters) {
        counters[0] += total.rho_floor; counters[1] += total.p_floor;
        counters[2] += total.newton_calls; counters[3] += total.newton_iters; counters[4] += total.newton_cap;
        counters[5] += total.bisect_calls; counters[6] += total.bisect_iters; counters[7] += total.bisect_cap;
        counters[8] += total.vacuum;
        if (total.newton_max > counters[9]) counters[9] = total.newton_max;
    }
    return T;
}

/*
 * Characteristic inflow at z_lo after a step (add2_bound, kernel.cu:1895-
 * 1925) with p_H = c->inflow_p and inflow speed c->inflow_v: column 0 of
 * (s2, u2) from the old column 0 of (s, u) and the new column 1 of (s2, u2).
 */
void ora_inflow(const ast_config* c, const double* s, const double* u, double* s2, double* u2)
{
    const int N = c->N, M = c->M;
    const double ggg = c->gamma, p_H = c->inflow_p, v_in = c->inflow_v;
    const d2* S = (const d2*)s;
    d2* S2 = (d2*)s2;
    d2* U2 = (d2*)u2;
    (void)u;
    for (int m = 0; m < M; m++) {
        const int index = m * N + 0;
        double pp2 = S2[(m)*N + 0 + 1].y;
        double uu2 = U2[(m)*N + 0 + 1].x;
        d2 s_do = S[index];
        double cc = sqrt(ggg * s_do.y / s_do.x);
        double T0 = p_H / (ggg - 1.0) / 1.0;
        double pp = pp2 - s_do.x * cc * (uu2 - v_in);
        double rho = pp / (ggg - 1.0) / T0;
        S2[index].x = rho;
        S2[index].y = p_H;
        U2[index].x = v_in;
        U2[index].y = 0.0;
    }
}

/*
 * nsteps steps in place on (s, u) with the reference's host protocol
 * (kernel.cu:3868-3947 + funk_time): each step uses *T_do, then
 * T_do <- new dt, TT += T_do, step += 1.
 */
int ora_run(const ast_config* c, double* s, double* u, int nsteps, double* T_do, double* TT,
            int64_t* step, int nthreads, int64_t* counters)
{
    size_t K = (size_t)c->N * (size_t)c->M;
    double* s2 = (double*)malloc(2 * K * sizeof(double));
    double* u2 = (double*)malloc(2 * K * sizeof(double));
    if (!s2 || !u2) { free(s2); free(u2); return -3; }
    for (int i = 0; i < nsteps; i++) {
        double T = ora_step(c, s, u, s2, u2, *T_do, nthreads, counters);
        if (c->inflow_p > 0.0) ora_inflow(c, s, u, s2, u2);
        *T_do = T;
        *TT = *TT + *T_do;
        *step = *step + 1;
        memcpy(s, s2, 2 * K * sizeof(double));
        memcpy(u, u2, 2 * K * sizeof(double));
    }
    free(s2);
    free(u2);
    return 0;
}

int ora_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
