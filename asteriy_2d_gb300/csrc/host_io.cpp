// host_io.cpp - configuration, initial conditions and the reference's file
// formats (host code of the C ABI).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <random>
#include <string>

#include "../../include/asteriy_gb300.h"

namespace {

// cell centres as the reference's writers compute them (kernel.cu:3127-3128,
// 4136-4137): x_min + n*(x_max-x_min)/(N-1), y_min + m*y_max/M
inline double out_x(const ast_config* c, int n) { return c->x_min + n * (c->x_max - c->x_min) / (c->N - 1); }
inline double out_y(const ast_config* c, int m)
{
    return (c->y_max / (2.0 * c->M)) + m * (c->y_max) / (c->M);
}
// cell centres as the kernels and the initial-condition loop compute them
// (kernel.cu:3345-3346): x_min + n*dx, y_min + m*dy
inline double cell_x(const ast_config* c, int n) { return c->x_min + n * ((c->x_max - c->x_min) / (c->N - 1)); }
inline double cell_y(const ast_config* c, int m) { return (c->y_max / (2.0 * c->M)) + m * ((c->y_max) / (c->M)); }

}  // namespace

extern "C" {

void ast_config_default(ast_config* c)
{
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->N = 32000;                       // Header.h:8
    c->M = 400;                         // Header.h:9
    c->x_min = 0.0;                     // Header.h:11
    c->x_max = 80.0;                    // Header.h:12
    c->y_max = 1.0;                     // Header.h:13
    c->gamma = 5.0 / 3.0;               // Header.h:17
    c->cfl = 0.05;                      // Header.h:47
    c->flux = AST_FLUX_HLL;
    c->recon = AST_RECON_MINMOD;
    c->geom = AST_GEOM_PLANAR;
    c->precision = AST_PREC_FP64;
    c->grad_p = 1;                      // Header.h:31
    c->guess = AST_GUESS_PVRS;
    c->bc[AST_Z_LO].kind = AST_BC_OUTFLOW;
    c->bc[AST_Z_HI].kind = AST_BC_OUTFLOW;
    c->bc[AST_R_LO].kind = AST_BC_REFLECT;
    c->bc[AST_R_HI].kind = AST_BC_REFLECT;
    c->fixed_az = c->fixed_ar = 1.0;
    c->riemann_max_iter = 200;
    c->dt_first = 0.000000001;          // kernel.cu:3322
    c->dt_cap = 1000;                   // kernel.cu:2530
    c->p_floor = 0.000001;              // kernel.cu:3072
    c->riemann_tol = 10e-10;            // Header.h:62
    c->mlp_gate = 0.2;
    c->inflow_v = 1.0;
    c->neutral_nh = 3.0;        // n_H, Header.h:85
    c->neutral_kn = 0.419231;   // Kn, Header.h:84
    c->persistent = 1;
}

int ast_config_check(const ast_config* c)
{
    if (!c) return AST_ERR_INVALID;
    if (c->N < 4 || c->M < 4 || (long long)c->N * c->M > (1LL << 31) - 1) return AST_ERR_INVALID;
    if (c->M > 65535 * 16) return AST_ERR_INVALID;
    if (!(c->x_max > c->x_min) || !(c->y_max > 0.0)) return AST_ERR_INVALID;
    if (!(c->gamma > 1.0) || !(c->cfl > 0.0)) return AST_ERR_INVALID;
    if (c->flux < AST_FLUX_HLL || c->flux > AST_FLUX_HLLCQ) return AST_ERR_INVALID;
    if (c->flux == AST_FLUX_HLLCQ && c->precision != AST_PREC_FP64) return AST_ERR_INVALID;
    if (c->recon < AST_RECON_NONE || c->recon > AST_RECON_MINMOD) return AST_ERR_INVALID;
    if (c->geom < AST_GEOM_PLANAR || c->geom > AST_GEOM_AXISYM) return AST_ERR_INVALID;
    if (c->precision < AST_PREC_FP64 || c->precision > AST_PREC_FP32) return AST_ERR_INVALID;
    if (c->guess < AST_GUESS_PVRS || c->guess > AST_GUESS_MLP) return AST_ERR_INVALID;
    if (c->copy_wait_polls < 0) return AST_ERR_INVALID;
    if (c->persistent < 0 || c->persistent > 2) return AST_ERR_INVALID;
    if (c->skip_uniform < 0 || c->skip_uniform > 1) return AST_ERR_INVALID;
    if (!(c->inflow_p >= 0.0)) return AST_ERR_INVALID;
    if (!std::isfinite(c->neutral_nh) || !std::isfinite(c->neutral_kn)) return AST_ERR_INVALID;
    for (int s = 0; s < 4; s++) {
        if (c->bc[s].kind < AST_BC_REFLECT || c->bc[s].kind > AST_BC_NONREFLECT) return AST_ERR_INVALID;
        if (c->bc[s].kind == AST_BC_FIXED && !(c->bc[s].rho > 0.0 && c->bc[s].p > 0.0)) return AST_ERR_INVALID;
    }
    if (c->fixed_region && !(c->fixed_az > 0.0 && c->fixed_ar > 0.0)) return AST_ERR_INVALID;
    if (c->riemann_max_iter < 1 || !(c->riemann_tol > 0.0)) return AST_ERR_INVALID;
    if (!(c->dt_first > 0.0) || !(c->dt_cap > 0.0) || !(c->p_floor > 0.0)) return AST_ERR_INVALID;
    return AST_OK;
}

int ast_fill_blast(const ast_config* c, double p_in, double p_out, double radius, double* s, double* u)
{
    if (!c || !s || !u || ast_config_check(c) != AST_OK) return AST_ERR_INVALID;
    for (int m = 0; m < c->M; m++) {
        for (int n = 0; n < c->N; n++) {
            const long long k = (long long)m * c->N + n;
            const double x = cell_x(c, n), y = cell_y(c, m);
            const double dist = std::sqrt(x * x + y * y);
            s[2 * k] = 1.0;
            s[2 * k + 1] = (dist < radius) ? p_in : p_out;
            u[2 * k] = 0.0;
            u[2 * k + 1] = 0.0;
        }
    }
    return AST_OK;
}

int ast_fill_wind(const ast_config* c, double r_w, double rho_w, double v_w, double mach_w, double rho_inf,
                  double p_inf, double v_inf, double noise, uint64_t seed, double* s, double* u)
{
    if (!c || !s || !u || ast_config_check(c) != AST_OK || !(r_w > 0.0)) return AST_ERR_INVALID;
    std::mt19937_64 gen(seed);
    const double p_w = rho_w * v_w * v_w / (c->gamma * mach_w * mach_w);
    for (int m = 0; m < c->M; m++) {
        for (int n = 0; n < c->N; n++) {
            const long long k = (long long)m * c->N + n;
            const double x = cell_x(c, n), y = cell_y(c, m);
            const double uni = (double)(gen() >> 11) * 0x1.0p-53;
            const double dist = std::sqrt(x * x + y * y);
            if (dist < r_w) {
                const double q = r_w / dist;
                s[2 * k] = rho_w * q * q;
                s[2 * k + 1] = p_w * std::pow(q, 2.0 * c->gamma);
                u[2 * k] = v_w * x / dist;
                u[2 * k + 1] = v_w * y / dist;
            } else {
                s[2 * k] = rho_inf * (1.0 + noise * (2.0 * uni - 1.0));
                s[2 * k + 1] = p_inf;
                u[2 * k] = v_inf;
                u[2 * k + 1] = 0.0;
            }
        }
    }
    return AST_OK;
}

// ---------------------------------------------------------------- problem sets
namespace {

inline double unit_draw(std::mt19937_64& gen) { return (double)(gen() >> 11) * 0x1.0p-53; }

void set_side(ast_config* c, int side, int kind, double rho = 0, double p = 0, double vz = 0, double vr = 0)
{
    c->bc[side].kind = kind;
    c->bc[side].rho = rho;
    c->bc[side].p = p;
    c->bc[side].vz = vz;
    c->bc[side].vr = vr;
}

// the blast / wind configurations of the single-problem benchmarks: z in
// [-1, 1], r in [0, 1], minmod, axisymmetric, CFL 0.4, reflecting axis
void base_config(ast_config* c, int N, int M, double gamma, int flux, int precision)
{
    ast_config_default(c);
    c->N = N;
    c->M = M;
    c->x_min = -1.0;
    c->x_max = 1.0;
    c->y_max = 1.0;
    c->gamma = gamma;
    c->cfl = 0.4;
    c->flux = flux;
    c->recon = AST_RECON_MINMOD;
    c->geom = AST_GEOM_AXISYM;
    c->precision = precision;
    set_side(c, AST_Z_LO, AST_BC_OUTFLOW);
    set_side(c, AST_Z_HI, AST_BC_OUTFLOW);
    set_side(c, AST_R_LO, AST_BC_REFLECT);
    set_side(c, AST_R_HI, AST_BC_OUTFLOW);
}

}  // namespace

int ast_problem_set(uint64_t seed, int nprob, int precision, ast_problem* out)
{
    if (!out || nprob < 1 || precision < AST_PREC_FP64 || precision > AST_PREC_FP32) return AST_ERR_INVALID;
    std::mt19937_64 gen(seed);
    for (int i = 0; i < nprob; i++) {
        ast_problem* P = &out[i];
        std::memset(P, 0, sizeof *P);
        const int M = (int)std::lround(64.0 * std::pow(8.0, unit_draw(gen)));
        P->mach = 1.5 + 4.5 * unit_draw(gen);
        const double gamma = (gen() >> 63) ? 1.4 : 5.0 / 3.0;
        P->setup = (gen() >> 63) ? AST_SETUP_WIND : AST_SETUP_BLAST;
        const int flux = (gen() >> 63) ? AST_FLUX_GODUNOV : AST_FLUX_HLLC;
        P->seed = gen();
        base_config(&P->cfg, 2 * M, M, gamma, flux, precision);
        if (P->setup == AST_SETUP_WIND) {
            // counterflow (rho 1, p 1/gamma: sound speed 1) entering at z = 1;
            // the wind sphere R < 0.05 at the origin is held fixed
            set_side(&P->cfg, AST_Z_HI, AST_BC_FIXED, 1.0, 1.0 / gamma, -P->mach, 0.0);
            P->cfg.fixed_region = 1;
            P->cfg.fixed_zc = 0.0;
            P->cfg.fixed_az = P->cfg.fixed_ar = 0.05;
        }
    }
    return AST_OK;
}

int ast_problem_fill(const ast_problem* P, double* s, double* u)
{
    if (!P || !s || !u) return AST_ERR_INVALID;
    const ast_config* c = &P->cfg;
    if (P->setup == AST_SETUP_BLAST) {
        const double g = c->gamma, m2 = P->mach * P->mach;
        const double p_out = 0.1, p_in = p_out * (2.0 * g * m2 - (g - 1.0)) / (g + 1.0);
        return ast_fill_blast(c, p_in, p_out, 0.2, s, u);
    }
    if (P->setup == AST_SETUP_WIND)
        return ast_fill_wind(c, 0.05, 1.0, 10.0, 10.0, 1.0, 1.0 / c->gamma, -P->mach, 0.01, P->seed, s, u);
    return AST_ERR_INVALID;
}

int ast_write_bin(const ast_config* c, const double* s, const double* u, const char* path)
{
    if (!c || !s || !u || !path || ast_config_check(c) != AST_OK) return AST_ERR_INVALID;
    std::ofstream f(path, std::ios::binary);
    if (!f) return AST_ERR_IO;
    for (int m = 0; m < c->M; m++) {
        for (int n = 0; n < c->N; n++) {
            const long long k = (long long)m * c->N + n;
            const double rec[6] = {out_x(c, n), out_y(c, m), s[2 * k], s[2 * k + 1], u[2 * k], u[2 * k + 1]};
            f.write(reinterpret_cast<const char*>(rec), sizeof rec);
        }
    }
    return f.good() ? AST_OK : AST_ERR_IO;
}

int ast_read_bin(const ast_config* c, double* s, double* u, const char* path)
{
    if (!c || !s || !u || !path || ast_config_check(c) != AST_OK) return AST_ERR_INVALID;
    std::ifstream f(path, std::ios::binary);
    if (!f) return AST_ERR_IO;
    const long long K = (long long)c->N * c->M;
    for (long long k = 0; k < K; k++) {
        double rec[6];
        f.read(reinterpret_cast<char*>(rec), sizeof rec);
        if (!f) return AST_ERR_IO;  // truncated file
        s[2 * k] = rec[2];
        s[2 * k + 1] = rec[3];
        u[2 * k] = rec[4];
        u[2 * k + 1] = rec[5];
    }
    return AST_OK;
}

int ast_write_tecplot(const ast_config* c, const double* s, const double* u, int stride, double soltime,
                      const char* path)
{
    if (!c || !s || !u || !path || stride < 1 || ast_config_check(c) != AST_OK) return AST_ERR_INVALID;
    std::ofstream f(path);
    if (!f) return AST_ERR_IO;
    const int N = c->N, M = c->M;
    const long long K = (long long)N * M;
    const double dx = (c->x_max - c->x_min) / (N - 1), dy = c->y_max / M;
    const int nn = (N + stride - 1) / stride, mm = (M + stride - 1) / stride;
    f << "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", \"Vx\", \"Vy\", \"Mach\", \"omega\", ZONE T = \"HP\", "
         "SOLUTIONTIME = "
      << soltime << ", N = " << nn * mm << " , E = " << (long long)(nn - 1) * (mm - 1)
      << ", F = FEPOINT, ET = quadrilateral" << std::endl;
    for (long long k = 0; k < K; k++) {
        const int n = (int)(k % N), m = (int)(k / N);
        if ((n % stride != 0) || (m % stride != 0)) continue;
        // neighbour indices as print_file_mini forms them (kernel.cu:3143-3152)
        const long long k2 = (long long)m * N + (n + 1), k3 = (long long)(m - 1) * N + n;
        const long long k4 = (long long)m * N + (n - 1), k5 = (long long)(m + 1) * N + n;
        double dvx = 0.0, dvy = 0.0, mach = 0.0;
        if (k3 >= 0 && k3 < K && k5 >= 0 && k5 < K) dvx = (u[2 * k5] - u[2 * k3]) / (2.0 * dy);
        if (k2 >= 0 && k2 < K && k4 >= 0 && k4 < K) dvy = (u[2 * k2 + 1] - u[2 * k4 + 1]) / (2.0 * dx);
        if (s[2 * k] > 0.0)
            mach = std::sqrt((u[2 * k] * u[2 * k] + u[2 * k + 1] * u[2 * k + 1]) / (c->gamma * s[2 * k + 1] / s[2 * k]));
        f << out_x(c, n) << " " << out_y(c, m) << " " << s[2 * k] << " " << s[2 * k + 1] << " " << u[2 * k] << " "
          << u[2 * k + 1] << " " << mach << " " << (dvy - dvx) / 2.0 << std::endl;
    }
    for (long long k = 0; k < (long long)nn * mm; k++) {
        const long long n = k % nn, m = k / nn;
        if ((m < mm - 1) && (n < nn - 1))
            f << m * nn + n + 1 << " " << m * nn + n + 2 << " " << (m + 1) * nn + n + 2 << " " << (m + 1) * nn + n + 1
              << std::endl;
    }
    return f.good() ? AST_OK : AST_ERR_IO;
}

int ast_write_tecplot_final(const ast_config* c, const double* s, const double* u, int stride, const char* path)
{
    if (!c || !s || !u || !path || stride < 1 || ast_config_check(c) != AST_OK) return AST_ERR_INVALID;
    std::ofstream f(path);
    if (!f) return AST_ERR_IO;
    const int N = c->N, M = c->M;
    const long long K = (long long)N * M;
    const double dx = (c->x_max - c->x_min) / (N - 1), dy = c->y_max / M;
    const int nn = (N + stride - 1) / stride, mm = (M + stride - 1) / stride;
    f << "TITLE = \"HP\"  VARIABLES = \"X\", \"Y\", \"Ro\", \"P\", \"Vx\", \"Vy\", \"Mach\", \"T\", \"Zav\", ZONE T = "
         "\"HP\", N = "
      << nn * mm << " , E = " << (long long)(nn - 1) * (mm - 1) << ", F = FEPOINT, ET = quadrilateral" << std::endl;
    for (long long k = 0; k < K; k++) {
        const int n = (int)(k % N), m = (int)(k / N);
        if ((n % stride != 0) || (m % stride != 0)) continue;
        double zav = 0.0;
        if (n > 0 && m > 0 && n < N - 1 && m < M - 1)
            zav = (u[2 * ((long long)m * N + n + 1) + 1] - u[2 * ((long long)m * N + n - 1) + 1]) / (2 * dx) -
                  (u[2 * ((long long)(m + 1) * N + n)] - u[2 * ((long long)(m - 1) * N + n)]) / (2 * dy);
        double mach = 0.0, temp = 0.0;
        if (s[2 * k] > 0.0) {
            mach = std::sqrt((u[2 * k] * u[2 * k] + u[2 * k + 1] * u[2 * k + 1]) / (c->gamma * s[2 * k + 1] / s[2 * k]));
            temp = s[2 * k + 1] / s[2 * k];
        }
        f << out_x(c, n) << " " << out_y(c, m) << " " << s[2 * k] << " " << s[2 * k + 1] << " " << u[2 * k] << " "
          << u[2 * k + 1] << " " << mach << " " << temp << " " << zav << std::endl;
    }
    for (long long k = 0; k < (long long)nn * mm; k++) {
        const long long n = k % nn, m = k / nn;
        if ((m < mm - 1) && (n < nn - 1))
            f << m * nn + n + 1 << " " << m * nn + n + 2 << " " << (m + 1) * nn + n + 2 << " " << (m + 1) * nn + n + 1
              << std::endl;
    }
    return f.good() ? AST_OK : AST_ERR_IO;
}

int ast_write_axis(const ast_config* c, const double* s, const double* u, const char* path)
{
    if (!c || !s || !u || !path || ast_config_check(c) != AST_OK) return AST_ERR_INVALID;
    std::ofstream f(path);
    if (!f) return AST_ERR_IO;
    for (int n = 0; n < c->N; n++) {
        const long long k = n;   // row m = 0
        double ss = 0.0;
        if (s[2 * k] > 0) ss = 1.0 / std::sqrt(c->gamma * s[2 * k + 1] / s[2 * k]);
        f << out_x(c, n) << " " << out_y(c, 0) << " " << s[2 * k] << " " << s[2 * k + 1] << " " << u[2 * k] << " "
          << u[2 * k + 1] << " " << ss << std::endl;
    }
    return f.good() ? AST_OK : AST_ERR_IO;
}

int ast_write_inform(const ast_config* c, double TT, double mach_inf, double chi, const char* path)
{
    if (!c || !path || ast_config_check(c) != AST_OK) return AST_ERR_INVALID;
    std::ofstream f(path);
    if (!f) return AST_ERR_IO;
    const long long K = (long long)c->N * c->M;
    f << "TT = " << TT << "    N = " << c->N << "   M = " << c->M << "   K = " << K << std::endl;
    f << "x_min = " << c->x_min << " " << "x_max = " << c->x_max << " " << "y_min = " << c->y_max / (2.0 * c->M) << " "
      << "y_max = " << c->y_max << std::endl;
    f << "M_inf = " << mach_inf << " " << "chi_ = " << chi << std::endl;
    return f.good() ? AST_OK : AST_ERR_IO;
}

}  // extern "C"
