// add2.cu - the drop-in for the reference's first-order planar step add2
// (kernel.cu:1928-2291), as its own kernel.
//
// add2 is not a special case of the face-once step: it evaluates each cell's
// four faces from that cell, and its flux selection is not symmetric.  The
// face on the cell's right and its r faces take HLLC inside the region
// (x + dx/2, resp. x, in (region_lo, region_hi)) and HLL outside, but the
// face on its left takes HLL inside the region (x - dx/2 in it) and HLLC
// outside (kernel.cu:2057-2085).  So inside the region the face between two
// cells is HLLC for the cell on its left and HLL for the cell on its right:
// the scheme is not conservative there.  This kernel reproduces that with
// one thread per cell evaluating its own four faces, as the reference does.
//
// Per cell (kernel.cu:1928-2291): neighbours with add2's boundary rules
// (right side outflow at n = N-1; left side the fixed inflow state at
// n = 0, its density perturbed by 1 + 0.01 sin(2 pi TT) for y < 0.5 while
// TT < 3 when method != 0; reflecting r = 0 and r = y_max); the four face
// fluxes (HLL or HLLC per the rule above, each in the cell's outward frame);
// dt candidate krit*rad/S per face; the planar update with the body force
// Q2 = -+amp*rho in v_r for body_lo < x < body_hi (r >= / < body_rsplit);
// the density and pressure floors.  *T is lowered to the cells' smallest dt
// candidate by an exact atomic minimum (the reference's write races).
#include <cuda_runtime.h>

#include "../../include/asteriy_gb300.h"
#include "launch.cuh"

using namespace ast;

namespace {

struct Add2Params {
    int N, M;
    double x_min, dx, y_min, dy;
    double krit_dx, krit_dy, dt_cap, p_floor;
    double region_lo, region_hi;
    int body_force;
    double body_lo, body_hi, body_rsplit, body_amp;
    double in_rho, in_p, in_vz, in_vr;   // the inflow state at n = 0 (the z_lo side's FIXED values)
    int perturb;                         // method != 0: the time-dependent inflow density
    Gas<double> g;
};

// the flux of the face with outward normal (n1, n2) between the cell (a)
// and its neighbour (b), in the cell's outward frame: returned as the
// outward mass and energy flux (ps) and the momentum flux vector (pu), and
// the face's wave speed; hllc selects the flux
__device__ __forceinline__ double add2_face(const Gas<double>& g, bool hllc, double2 sa, double2 ua, double2 sb,
                                            double2 ub, double n1, double n2, double2& ps, double2& pu)
{
    // tangent t = (-n2, n1); normal and tangential velocities of each side
    const double unA = ua.x * n1 + ua.y * n2, utA = -ua.x * n2 + ua.y * n1;
    const double unB = ub.x * n1 + ub.y * n2, utB = -ub.x * n2 + ub.y * n1;
    double F[4];
    const double S = hllc ? flux_hllc(g, sa.x, sa.y, unA, utA, sb.x, sb.y, unB, utB, F)
                          : flux_hll(g, sa.x, sa.y, unA, utA, sb.x, sb.y, unB, utB, F);
    ps = make_double2(F[0], F[3]);
    pu = make_double2(F[1] * n1 - F[2] * n2, F[1] * n2 + F[2] * n1);
    return S;
}

__device__ __forceinline__ bool in_region(const Add2Params& P, double xf)
{
    return xf > P.region_lo && xf < P.region_hi;
}

__global__ void add2_kernel(const double2* __restrict__ s, const double2* __restrict__ u, double2* s2, double2* u2,
                            double* T, const double* T_do_p, const double* TT_p, Add2Params P)
{
    const long long index = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (index >= (long long)P.N * P.M) return;
    const int N = P.N, M = P.M;
    const int n = (int)(index % N), m = (int)(index / N);
    // cell centres as the reference forms them (separate products and sums)
    const double y = __dadd_rn(P.y_min, __dmul_rn((double)m, P.dy));
    const double x = __dadd_rn(P.x_min, __dmul_rn((double)n, P.dx));
    const double2 s1 = s[index], u1 = u[index];
    double2 sR, uR, sL, uL, sT, uT, sB, uB;
    // right (kernel.cu:1971-2001): outflow copy at n = N-1
    if (n == N - 1) { sR = s1; uR = u1; }
    else { sR = s[index + 1]; uR = u[index + 1]; }
    // left (kernel.cu:2004-2024): the fixed inflow state at n = 0
    if (n == 0) {
        sL = make_double2(P.in_rho, P.in_p);
        uL = make_double2(P.in_vz, P.in_vr);
        const double TT = *TT_p;
        if (y < 0.5 && TT < 3.0 && P.perturb) sL.x = sL.x * (1.0 + 0.01 * sin(TT * 3.14159265358979323846 * 2.0));
    } else {
        sL = s[index - 1];
        uL = u[index - 1];
    }
    // top (kernel.cu:2026-2036) and bottom (2044-2054): reflecting
    if (m == M - 1) { sT = s1; uT = make_double2(u1.x, -u1.y); }
    else { sT = s[index + N]; uT = u[index + N]; }
    if (m == 0) { sB = s1; uB = make_double2(u1.x, -u1.y); }
    else { sB = s[index - N]; uB = u[index - N]; }

    const Gas<double>& g = P.g;
    double2 Ps12, Pu12, Ps13, Pu13, Ps14, Pu14, Ps15, Pu15;
    const double hdx = P.dx / 2.0;
    const double S12 = add2_face(g, in_region(P, x + hdx), s1, u1, sR, uR, 1.0, 0.0, Ps12, Pu12);
    const bool rr = in_region(P, x);
    const double S13 = add2_face(g, rr, s1, u1, sB, uB, 0.0, -1.0, Ps13, Pu13);
    const double S15 = add2_face(g, rr, s1, u1, sT, uT, 0.0, 1.0, Ps15, Pu15);
    // the left face: HLL inside the region, HLLC outside (kernel.cu:2078-2085)
    const double S14 = add2_face(g, !in_region(P, x - hdx), s1, u1, sL, uL, -1.0, 0.0, Ps14, Pu14);
    // dt candidate: min over faces of krit*rad/S = krit*rad/max S
    const double sz = fmax(S12, S14), sr = fmax(S13, S15);
    double tmin = P.dt_cap;
    if (sz > 0.0) tmin = fmin(tmin, P.krit_dx / sz);
    if (sr > 0.0) tmin = fmin(tmin, P.krit_dy / sr);
    atomicMin((unsigned long long*)T, (unsigned long long)__double_as_longlong(tmin));

    // the planar update (kernel.cu:2201-2290)
    const double dy = P.dy, dx = P.dx;
    const double PSx = (Ps12.x + Ps14.x) * dy + (Ps13.x + Ps15.x) * dx;
    const double PSy = (Ps12.y + Ps14.y) * dy + (Ps13.y + Ps15.y) * dx;
    const double PUx = (Pu12.x + Pu14.x) * dy + (Pu13.x + Pu15.x) * dx;
    const double PUy = (Pu12.y + Pu14.y) * dy + (Pu13.y + Pu15.y) * dx;
    const double dV = dx * dy;
    double Q2 = 0.0;
    if (P.body_force && x > P.body_lo && x < P.body_hi) Q2 = (y >= P.body_rsplit) ? -P.body_amp * s1.x : P.body_amp * s1.x;
    const double Q3 = Q2 * u1.y;
    const double T_do = *T_do_p;
    const double tdv = T_do / dV;
    double rho2 = s1.x - tdv * PSx;
    if (rho2 <= 0.0) rho2 = s1.x;
    const double vz2 = (s1.x * u1.x - tdv * PUx) / rho2;
    const double vr2 = (s1.x * u1.y - tdv * PUy + T_do * Q2) / rho2;
    const double g1 = g.g1;
    double p2 = (((s1.y / g1 + s1.x * (u1.x * u1.x + u1.y * u1.y) * 0.5) - tdv * PSy + T_do * Q3) -
                 0.5 * rho2 * (vz2 * vz2 + vr2 * vr2)) *
                g1;
    if (p2 <= 0.0) p2 = P.p_floor;
    s2[index] = make_double2(rho2, p2);
    u2[index] = make_double2(vz2, vr2);
}

}  // namespace

extern "C" int ast_add2_raw(const double* s, const double* u, double* s2, double* u2, double* T, const double* T_do,
                            const double* TT, int method, int step, const ast_config* cfg, void* stream)
{
    (void)step;
    if (!s || !u || !s2 || !u2 || !T || !T_do || !TT || !cfg) return set_error(AST_ERR_INVALID, "null argument");
    int rc = ast_config_check(cfg);
    if (rc != AST_OK) return rc;
    if (cfg->precision != AST_PREC_FP64 || cfg->recon != AST_RECON_NONE || cfg->geom != AST_GEOM_PLANAR ||
        cfg->bc[AST_Z_LO].kind != AST_BC_FIXED)
        return set_error(AST_ERR_INVALID, "add2 is FP64, first order, planar, with a fixed z_lo inflow");
    Add2Params P;
    P.N = cfg->N;
    P.M = cfg->M;
    P.x_min = cfg->x_min;
    P.dx = (cfg->x_max - cfg->x_min) / (cfg->N - 1);
    P.dy = cfg->y_max / cfg->M;
    P.y_min = cfg->y_max / (2.0 * cfg->M);
    P.krit_dx = cfg->cfl * P.dx;
    P.krit_dy = cfg->cfl * P.dy;
    P.dt_cap = cfg->dt_cap;
    P.p_floor = cfg->p_floor;
    P.region_lo = cfg->region_select ? cfg->region_lo : 1e300;
    P.region_hi = cfg->region_select ? cfg->region_hi : -1e300;
    P.body_force = cfg->body_force;
    P.body_lo = cfg->body_lo;
    P.body_hi = cfg->body_hi;
    P.body_rsplit = cfg->body_rsplit;
    P.body_amp = cfg->body_amp;
    P.in_rho = cfg->bc[AST_Z_LO].rho;
    P.in_p = cfg->bc[AST_Z_LO].p;
    P.in_vz = cfg->bc[AST_Z_LO].vz;
    P.in_vr = cfg->bc[AST_Z_LO].vr;
    P.perturb = method != 0;
    P.g = make_gas<double>(cfg->gamma, cfg->riemann_tol, cfg->riemann_max_iter);
    const long long K = (long long)cfg->N * cfg->M;
    add2_kernel<<<(unsigned)((K + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        (const double2*)s, (const double2*)u, (double2*)s2, (double2*)u2, T, T_do, TT, P);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "add2 kernel launch");
}
