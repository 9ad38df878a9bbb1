/*
 * ref_shim.h - host environment in which the reference's own device
 * functions compile as plain C++ (TEST INFRASTRUCTURE ONLY).
 *
 * oracle/make_ref.py copies selected functions of the reference, unchanged,
 * into oracle/_ref/ref_extract.inc (git-ignored, never committed).
 * oracle/ref_driver.cpp includes this header, then that file, and drives
 * the reference's step kernels cell by cell from an OpenMP loop.
 *
 * What this header provides:
 *   - CUDA qualifiers as empty macros, host double2/double3, thread-local
 *     threadIdx/blockIdx/blockDim so that `index` equals the cell index;
 *   - min/max on doubles with CUDA's semantics (fmin/fmax);
 *   - __dsqrt_rn as the correctly rounded sqrt;
 *   - the reference's Header.h parameters (Header.h:6-70) as runtime
 *     variables, so one build serves any grid, gamma and CFL.  The derived
 *     constants (g1, g2, gp, gm, ...) are defined by the same formulas as
 *     Header.h:20-26 so that they round identically.
 * The standard headers come first: the reference's single-letter macros
 * (N, M, K) would otherwise collide with library identifiers.
 */
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <string>

struct ref_uint3 { unsigned int x, y, z; };
extern thread_local ref_uint3 threadIdx, blockIdx, blockDim;

struct double2 { double x, y; };
struct double3 { double x, y, z; };

static inline double min(double a, double b) { return std::fmin(a, b); }
static inline double max(double a, double b) { return std::fmax(a, b); }
static inline double __dsqrt_rn(double v) { return std::sqrt(v); }

/* diagnostics printed by the reference are counted, not printed */
int ref_printf(const char* fmt, ...);

extern int ref_N, ref_M;
extern double ref_x_min, ref_x_max, ref_y_max, ref_gamma, ref_krit;

#define __device__
#define __global__
#define __host__
#define printf ref_printf

#define N ref_N
#define M ref_M
#define K (N * M)
#define x_min ref_x_min
#define x_max ref_x_max
#define y_max ref_y_max
#define y_min (y_max / (2.0 * M))
#define dx ((x_max - x_min) / (N - 1))
#define dy ((y_max) / (M))
#define ggg ref_gamma
#define ga ref_gamma
#define gga ga
#define g1 (ga - 1.0)
#define gg1 (ga - 1.0)
#define g2 (ga + 1.0)
#define gg2 (ga + 1.0)
#define gp ((g2 / ga) / 2.0)
#define gm ((g1 / ga) / 2.0)
#define krit ref_krit
#define kv(x) ((x) * (x))
#define eps 10e-10
#define eps8 10e-8
#define pi 3.14159265358979323846
#define p_H 7.0
#define Omega 0.0
#define hx -100.4
#define hy -1.0
#define grad_p true
#define Velosity_inf -2.54186
#define n_H 3.0
#define Kn 0.419231
