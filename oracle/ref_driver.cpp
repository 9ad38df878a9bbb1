/*
 * ref_driver.cpp - drives the reference's own functions on the host
 * (TEST INFRASTRUCTURE ONLY; used to pin the oracle and to generate the
 * golden vectors under tests/golden/).
 *
 * The reference code itself is not in this file: it is included from
 * oracle/_ref/ref_extract.inc, which oracle/make_ref.py extracts unchanged
 * from the reference sources.  This file only supplies a loop over cells,
 * the exact minimum of the per-cell dt the reference races on
 * (kernel.cu:3013-3017), and C entry points for ctypes.
 */
#include "ref_shim.h"

#include "_ref/ref_extract.inc"

#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

thread_local ref_uint3 threadIdx, blockIdx, blockDim;
int ref_N = 64, ref_M = 32;
double ref_x_min = 0.0, ref_x_max = 80.0, ref_y_max = 1.0;
double ref_gamma = 5.0 / 3.0, ref_krit = 0.05;
static long long g_diag = 0;

#undef printf
int ref_printf(const char*, ...)
{
#ifdef _OPENMP
#pragma omp atomic
#endif
    g_diag++;
    return 0;
}

extern "C" {

void ref_set_params(int n_, int m_, double xmin, double xmax, double ymax, double gamma, double cfl)
{
    ref_N = n_; ref_M = m_;
    ref_x_min = xmin; ref_x_max = xmax; ref_y_max = ymax;
    ref_gamma = gamma; ref_krit = cfl;
}

long long ref_diag_count(void) { return g_diag; }

double ref_minmod(double a, double b) { return minmod(a, b); }

double ref_linear(double x1, double t1, double x2, double t2, double x3, double t3, double y)
{
    return linear(x1, t1, x2, t2, x3, t3, y);
}

void ref_linear2(double x1, double t1, double x2, double t2, double x3, double t3,
                 double y1, double y2, double* A, double* B)
{
    linear2(x1, t1, x2, t2, x3, t3, y1, y2, *A, *B);
}

/* which: 0 HLL, 1 HLLC (nul_potok=false), 2 exact Godunov,
          3 HLLC_Aleksashov, 4 HLLC (nul_potok=true), 5 HLLCQ_Korolkov_2D
          (its passive scalar zero).
   out[4] = (mass, mom_z, mom_r, energy); returns the face dt. */
double ref_face(int which, const double* sL, const double* uL, const double* sR, const double* uR,
                double n1, double n2, double rad, double* out)
{
    double2 Ls = {sL[0], sL[1]}, Lu = {uL[0], uL[1]}, Rs = {sR[0], sR[1]}, Ru = {uR[0], uR[1]};
    double2 Ps = {0, 0}, Pu = {0, 0};
    double t = 0.0;
    switch (which) {
    case 0: t = HLL(Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad); break;
    case 1: t = HLLC_2d_Korolkov(Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad, false); break;
    case 2: t = Godunov_Solver_Alexashov(Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad); break;
    case 3: t = HLLC_Aleksashov(Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad); break;
    case 4: t = HLLC_2d_Korolkov(Ls, Lu, Rs, Ru, n1, n2, Ps, Pu, rad, true); break;
    case 5: {
        double PQ = 0.0;
        t = HLLCQ_Korolkov_2D(Ls, Lu, Rs, Ru, 0.0, 0.0, n1, n2, Ps, Pu, PQ, rad);
        break;
    }
    default: return -1.0;
    }
    out[0] = Ps.x; out[1] = Pu.x; out[2] = Pu.y; out[3] = Ps.y;
    return t;
}

/* A face with a passive scalar Q (QL, QR on the two sides).  which: 1 HLLC
   (HLLC_2d_Korolkov_b_s, metod 2, W = 0, nul_potok = false, its PQ), 5
   HLLCQ_Korolkov_2D.  out[5] = (mass, mom_z, mom_r, energy, PQ); returns the
   face dt. */
double ref_face_q(int which, const double* sL, const double* uL, const double* sR, const double* uR, double QL,
                  double QR, double n1, double n2, double rad, double* out)
{
    double2 Ls = {sL[0], sL[1]}, Lu = {uL[0], uL[1]}, Rs = {sR[0], sR[1]}, Ru = {uR[0], uR[1]};
    double2 Ps = {0, 0}, Pu = {0, 0};
    double PQ = 0.0, t = 0.0;
    if (which == 5) {
        t = HLLCQ_Korolkov_2D(Ls, Lu, Rs, Ru, QL, QR, n1, n2, Ps, Pu, PQ, rad);
        out[0] = Ps.x; out[1] = Pu.x; out[2] = Pu.y; out[3] = Ps.y;
    } else if (which == 1) {
        double P[4] = {0, 0, 0, 0}, Vl, Vc, Vp;
        t = HLLC_2d_Korolkov_b_s(Ls.x, QL, Ls.y, Lu.x, Lu.y, Rs.x, QR, Rs.y, Ru.x, Ru.y, 0.0, P, PQ, n1, n2, rad, 2,
                                 Vl, Vc, Vp, false);
        out[0] = P[0]; out[1] = P[1]; out[2] = P[2]; out[3] = P[3];
    } else {
        return -1.0;
    }
    out[4] = PQ;
    return t;
}

/* nn2 of add_MK's launches (K double3), or NULL for the zeros of the
   reference's main (kernel.cu:3338). */
static const double3* g_ref_nn2 = nullptr;

void ref_set_neutral(const double* nn2) { g_ref_nn2 = reinterpret_cast<const double3*>(nn2); }

/*
 * One launch of a reference step kernel over all K cells.
 * kernel: 0 Kernel_TVD (kernel.cu:2513), 1 add_MK (kernel.cu:2293),
 *         2 add2 (kernel.cu:1928).
 * s, u, s2, u2: K (x, y) pairs.  Returns min(1e7, every cell's tmin),
 * i.e. *T after the launch with T reset to 1e7 before it.
 */
double ref_kernel_step(int kernel, const double* s, const double* u, double* s2, double* u2,
                       double T_do, double TT, int method, int nthreads)
{
    const int Kc = ref_N * ref_M;
    double2* S = (double2*)s;
    double2* U = (double2*)u;
    double2* S2 = (double2*)s2;
    double2* U2 = (double2*)u2;
    std::vector<double> nn1(Kc, 0.0), nn3(Kc, 0.0);
    std::vector<double3> nn2(Kc, double3{0.0, 0.0, 0.0});
    double T = 10000000;
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nthreads)
#endif
    {
        double Tl = 10000000;
        double Tdo = T_do, TTl = TT;
        blockIdx.x = 0;
        blockDim.x = 1;
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int k = 0; k < Kc; k++) {
            threadIdx.x = (unsigned int)k;
            if (kernel == 0) Kernel_TVD(S, U, S2, U2, &Tl, &Tdo, &TTl, method);
            else if (kernel == 1)
                add_MK(S, U, S2, U2, nn1.data(), g_ref_nn2 ? const_cast<double3*>(g_ref_nn2) : nn2.data(),
                       nn3.data(), &Tl, &Tdo, method, 0);
            else add2(S, U, S2, U2, &Tl, &Tdo, &TTl, method, 0);
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            if (T > Tl) T = Tl;
        }
    }
    return T;
}

/* One launch of the reference's add2_bound (kernel.cu:1895-1925) over all K
   cells on (s, u) -> (s2, u2); p_H is the shim's 7. */
void ref_bound(const double* s, const double* u, double* s2, double* u2)
{
    const int Kc = ref_N * ref_M;
    double T = 10000000, Tdo = 0.0, TTl = 0.0;
    blockIdx.x = 0;
    blockDim.x = 1;
    for (int k = 0; k < Kc; k++) {
        threadIdx.x = (unsigned int)k;
        add2_bound((double2*)s, (double2*)u, (double2*)s2, (double2*)u2, &T, &Tdo, &TTl, 1, 0);
    }
}

/* nsteps launches with the host protocol of kernel.cu:3868-3947 and
   funk_time (kernel.cu:1525-1536), in place on s, u. */
int ref_kernel_run(int kernel, double* s, double* u, int nsteps, int method, double* T_do,
                   double* TT, long long* step, int nthreads)
{
    const size_t Kc = (size_t)ref_N * ref_M;
    std::vector<double> s2(2 * Kc), u2(2 * Kc);
    for (int i = 0; i < nsteps; i++) {
        double T = ref_kernel_step(kernel, s, u, s2.data(), u2.data(), *T_do, *TT, method, nthreads);
        *T_do = T;
        *TT = *TT + *T_do;
        *step = *step + 1;
        std::memcpy(s, s2.data(), 2 * Kc * sizeof(double));
        std::memcpy(u, u2.data(), 2 * Kc * sizeof(double));
    }
    return 0;
}

int ref_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} /* extern "C" */
