// launch.cuh - launch helpers of the step kernels.  The instantiations are
// spread over several translation units (step_f64.cu, step_f32.cu,
// step_raw.cu, batch_f64_s*.cu, batch_f32_s*.cu) so that they compile in
// parallel.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <climits>
#include <cmath>
#include <cstring>

#include <algorithm>

#include "../../include/asteriy_gb300.h"
#include "step.cuh"
#include "sweep.cuh"

namespace ast {

constexpr int kTZ = 32, kTR = 16;
static_assert(kTZ == kTmaTZ && kTR == kTmaTR, "the persistent kernels' tile is the solver's tile");

// records the failure text for ast_last_error() and returns AST_ERR_CUDA
int cuda_fail(cudaError_t e, const char* what);
// records msg for ast_last_error() and returns code
int set_error(int code, const char* msg);
// writes the packed network after the parameter block W (device, kMlpDevFloats
// floats) on stream st
int launch_mlp_pack(float* W, cudaStream_t st);

// the four FP32 state planes of one time level (base, rows of ld, planes
// of `plane` elements) as a 3-D tensor map with a box of bx x by x 4
int encode_planes(CUtensorMap* map, void* base, const ast_config& c, long long ld, long long plane, unsigned bx,
                  unsigned by);

// the SM count of the current device (looked up once per device)
inline int sm_count()
{
    constexpr int kMaxDev = 64;
    static int n[kMaxDev] = {};
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev >= 0 && dev < kMaxDev && n[dev] > 0) return n[dev];
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return 1;
    if (dev >= 0 && dev < kMaxDev) n[dev] = v;
    return v;
}

// launch=false only raises the kernel's dynamic shared-memory limit, which
// must happen outside stream capture (ast_create, ast_step_raw).  The FP64
// solver on a small grid (fewer 32x16 tiles than two per SM) steps with
// 16x16 tiles: twice the CTAs with half the cells each, since there every
// CTA runs alone on its SM at the FP64 rate.  P.band_hi > 0 launches the
// tile rows [band_lo, band_hi) only (both tile shapes are 16 rows high), and
// every tile of the grid counts towards the step's clock.
template <typename R, int FLUX, bool RECON, int LAYOUT>
int launch_step_t(const StepParams& P, cudaStream_t st, bool launch)
{
    constexpr bool kSmallTiles = sizeof(R) == 8;
    constexpr int kSZ = 16, kSR = 16;
    auto k = step_kernel<R, FLUX, RECON, LAYOUT, kTZ, kTR>;
    constexpr size_t smem = tile_smem_bytes<R, FLUX, kTZ, kTR>();
    cudaError_t e;
    if (!launch) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
        if constexpr (kSmallTiles) {
            e = cudaFuncSetAttribute(step_kernel<R, FLUX, RECON, LAYOUT, kSZ, kSR>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)tile_smem_bytes<R, FLUX, kSZ, kSR>());
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
        }
        return AST_OK;
    }
    static_assert(kSR == kTR, "bands are counted in tile rows of either shape");
    const int rows = (P.M + kTR - 1) / kTR;
    const int band = P.band_hi > 0 ? P.band_hi - P.band_lo : rows;
    StepParams Q = P;
    const long long tiles = (long long)((P.N + kTZ - 1) / kTZ) * rows;
    if constexpr (kSmallTiles) {
        if (tiles < 2LL * sm_count()) {
            dim3 grid((P.N + kSZ - 1) / kSZ, band);
            if (P.band_hi > 0) Q.units = (int)grid.x * rows;
            step_kernel<R, FLUX, RECON, LAYOUT, kSZ, kSR>
                <<<grid, kThreads, tile_smem_bytes<R, FLUX, kSZ, kSR>(), st>>>(Q);
            e = cudaGetLastError();
            return e == cudaSuccess ? AST_OK : cuda_fail(e, "step kernel launch");
        }
    }
    dim3 grid((P.N + kTZ - 1) / kTZ, band);
    if (P.band_hi > 0) Q.units = (int)grid.x * rows;
    k<<<grid, kThreads, smem, st>>>(Q);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "step kernel launch");
}

// the persistent kernel (FP32 or FP64 state planes) over `grid` CTAs;
// launch=false raises its shared-memory limit and returns the CTAs per SM it
// reaches in *per_sm
template <typename R, int FLUX, bool RECON>
int launch_tma_t(const StepParams& P, const CUtensorMap& tin, const CUtensorMap& tout, int grid, cudaStream_t st,
                 bool launch, int* per_sm)
{
    // two variants: with the uniform-tile test (skip_uniform) and without it
    auto k = P.skip_uniform ? step_kernel_tma<R, FLUX, RECON, true> : step_kernel_tma<R, FLUX, RECON, false>;
    constexpr size_t smem = tile_smem_bytes<R, FLUX, kTmaTZ, kTmaTR, 2>();
    cudaError_t e;
    if (!launch) {
        for (auto kv : {step_kernel_tma<R, FLUX, RECON, true>, step_kernel_tma<R, FLUX, RECON, false>}) {
            e = cudaFuncSetAttribute(kv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
        }
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, kThreads, smem);
        return e == cudaSuccess ? AST_OK : cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    }
    k<<<grid, kThreads, smem, st>>>(P, tin, tout);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "persistent step kernel launch");
}

int launch_step_tma(const StepParams& P, const CUtensorMap& tin, const CUtensorMap& tout, int flux, int recon,
                    int grid, cudaStream_t st, bool launch, int* per_sm);
// the same for FP64 state planes (the FP64 solver on grids of at least two
// 32x16 tiles per SM)
int launch_step_tma64(const StepParams& P, const CUtensorMap& tin, const CUtensorMap& tout, int flux, int recon,
                      int grid, cudaStream_t st, bool launch, int* per_sm);
inline int launch_step_tma_e(size_t elem, const StepParams& P, const CUtensorMap& tin, const CUtensorMap& tout,
                             int flux, int recon, int grid, cudaStream_t st, bool launch, int* per_sm)
{
    return elem == 8 ? launch_step_tma64(P, tin, tout, flux, recon, grid, st, launch, per_sm)
                     : launch_step_tma(P, tin, tout, flux, recon, grid, st, launch, per_sm);
}

// the FP32 strip kernel over `grid` CTAs; launch=false returns the CTAs per
// SM it reaches in *per_sm
template <int FLUX, bool RECON>
int launch_sweep_t(const StepParams& P, int grid, cudaStream_t st, bool launch, int* per_sm)
{
    auto k = sweep_kernel<FLUX, RECON>;
    cudaError_t e;
    if (!launch) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, kThreads, 0);
        return e == cudaSuccess ? AST_OK : cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    }
    k<<<grid, kThreads, 0, st>>>(P);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "strip kernel launch");
}

// the FP32 strip kernel of a flux and reconstruction
int launch_step_sweep(const StepParams& P, int flux, int recon, int grid, cudaStream_t st, bool launch, int* per_sm);
// strips of the strip kernel in tile rows [band_lo, band_hi) (all rows when
// band_hi is 0) of an N x M grid
inline int sweep_strips(int N, int M, int band_lo, int band_hi)
{
    const int r_lo = band_lo * kTR, r_hi = band_hi > 0 ? std::min(band_hi * kTR, M) : M;
    return ((N + kSW - 1) / kSW) * ((r_hi - r_lo + kSH - 1) / kSH);
}

// the persistent FP32 batch kernel (one class, or MIXED: every problem)
// over `total` work-list entries with `grid` CTAs; its problems are the
// slots [slot0, slot0 + nslots) (maps and parameters in device memory,
// indexed by slot; counter[0..1] zero before the first launch, rewound by
// each launch); launch=false raises its shared-memory limit and returns the
// CTAs per SM it reaches in *per_sm
template <int FLUX, bool RECON, bool MIXED>
int launch_batch_tma_t(const StepParams* Ps, const CUtensorMap* tin, const CUtensorMap* tout, const BatchTile* work,
                       int total, int slot0, int nslots, unsigned int* counter, int wait_polls, int grid,
                       cudaStream_t st, bool launch, int* per_sm)
{
    auto k = batch_kernel_tma<FLUX, RECON, MIXED>;
    constexpr size_t smem = tile_smem_bytes<float, MIXED ? 2 : FLUX, kTmaTZ, kTmaTR, 2>();
    cudaError_t e;
    if (!launch) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, kThreads, smem);
        return e == cudaSuccess ? AST_OK : cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    }
    if (grid <= 0 || total <= 0) return AST_OK;
    k<<<grid, kThreads, smem, st>>>(Ps, tin, tout, work, total, slot0, nslots, counter, wait_polls);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "persistent batch kernel launch");
}

int launch_batch_tma(const StepParams* Ps, const CUtensorMap* tin, const CUtensorMap* tout, const BatchTile* work,
                     int total, int slot0, int nslots, unsigned int* counter, int wait_polls, int flux, int recon,
                     int grid, cudaStream_t st, bool launch, int* per_sm);

template <typename R, int LAYOUT>
int launch_step_r(const StepParams& P, int flux, int recon, cudaStream_t st, bool launch)
{
    if (flux == AST_FLUX_HLLCQ) {
        // HLLCQ_Korolkov_2D: FP64 only
        if constexpr (sizeof(R) == 8)
            return recon ? launch_step_t<R, 4, true, LAYOUT>(P, st, launch)
                         : launch_step_t<R, 4, false, LAYOUT>(P, st, launch);
        else
            return set_error(AST_ERR_UNSUPPORTED, "HLLCQ is an FP64 flux");
    }
    if (recon) {
        if (flux == AST_FLUX_HLL) return launch_step_t<R, 0, true, LAYOUT>(P, st, launch);
        if (flux == AST_FLUX_HLLC) return launch_step_t<R, 1, true, LAYOUT>(P, st, launch);
        if (flux == AST_FLUX_HLLC_A) return launch_step_t<R, 3, true, LAYOUT>(P, st, launch);
        return launch_step_t<R, 2, true, LAYOUT>(P, st, launch);
    }
    if (flux == AST_FLUX_HLL) return launch_step_t<R, 0, false, LAYOUT>(P, st, launch);
    if (flux == AST_FLUX_HLLC) return launch_step_t<R, 1, false, LAYOUT>(P, st, launch);
    if (flux == AST_FLUX_HLLC_A) return launch_step_t<R, 3, false, LAYOUT>(P, st, launch);
    return launch_step_t<R, 2, false, LAYOUT>(P, st, launch);
}

// tile shapes of the batch kernels (the autotuner's choices): z x r cells
constexpr int kNumShapes = 3;
constexpr int kShapeTZ[kNumShapes] = {32, 16, 64};
constexpr int kShapeTR[kNumShapes] = {16, 16, 8};

// the batch kernel of one (flux, recon) class over `tiles` work-list entries
template <typename R, int FLUX, bool RECON, int TZ, int TR>
int launch_batch_t(const StepParams* Ps, const int* tile_start, int nprob, int tiles, cudaStream_t st, bool launch)
{
    auto k = batch_kernel<R, FLUX, RECON, TZ, TR>;
    constexpr size_t smem = tile_smem_bytes<R, FLUX, TZ, TR>();
    cudaError_t e;
    if (!launch) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return e == cudaSuccess ? AST_OK : cuda_fail(e, "cudaFuncSetAttribute");
    }
    k<<<tiles, kThreads, smem, st>>>(Ps, tile_start, nprob);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "batch kernel launch");
}

template <typename R, int TZ, int TR>
int launch_batch_r(const StepParams* Ps, const int* tile_start, int nprob, int tiles, int flux, int recon,
                   cudaStream_t st, bool launch)
{
    if (recon) {
        if (flux == AST_FLUX_HLL) return launch_batch_t<R, 0, true, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
        if (flux == AST_FLUX_HLLC) return launch_batch_t<R, 1, true, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
        if (flux == AST_FLUX_HLLC_A)
            return launch_batch_t<R, 3, true, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
        return launch_batch_t<R, 2, true, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
    }
    if (flux == AST_FLUX_HLL) return launch_batch_t<R, 0, false, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
    if (flux == AST_FLUX_HLLC) return launch_batch_t<R, 1, false, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
    if (flux == AST_FLUX_HLLC_A) return launch_batch_t<R, 3, false, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
    return launch_batch_t<R, 2, false, TZ, TR>(Ps, tile_start, nprob, tiles, st, launch);
}

#define AST_BATCH_EXTERN(R, S)                                                                          \
    extern template int launch_batch_r<R, kShapeTZ[S], kShapeTR[S]>(const StepParams*, const int*, int, int, \
                                                                    int, int, cudaStream_t, bool);
AST_BATCH_EXTERN(double, 0)
AST_BATCH_EXTERN(double, 1)
AST_BATCH_EXTERN(double, 2)
AST_BATCH_EXTERN(float, 0)
AST_BATCH_EXTERN(float, 1)
AST_BATCH_EXTERN(float, 2)
#undef AST_BATCH_EXTERN

// a batch class launch in precision `elem` (bytes) with tile shape `shape`
inline int launch_batch(size_t elem, int shape, const StepParams* Ps, const int* tile_start, int nprob, int tiles,
                        int flux, int recon, cudaStream_t st, bool launch)
{
#define AST_BATCH_CASE(R, S)                                                                             \
    return launch_batch_r<R, kShapeTZ[S], kShapeTR[S]>(Ps, tile_start, nprob, tiles, flux, recon, st, launch)
    if (elem == 8) {
        if (shape == 1) AST_BATCH_CASE(double, 1);
        if (shape == 2) AST_BATCH_CASE(double, 2);
        AST_BATCH_CASE(double, 0);
    }
    if (shape == 1) AST_BATCH_CASE(float, 1);
    if (shape == 2) AST_BATCH_CASE(float, 2);
    AST_BATCH_CASE(float, 0);
#undef AST_BATCH_CASE
}

// the FP32 batch kernel over problems of every flux (32x16 tiles, one
// reconstruction) over `tiles` work-list entries; launch=false raises its
// shared-memory limit
int launch_batch_mixed(const StepParams* Ps, const int* tile_start, const int* flux_of, int nprob, int tiles,
                       int recon, cudaStream_t st, bool launch);

// the one-launch persistent FP32 batch kernel (every problem, one
// reconstruction), as launch_batch_tma
int launch_batch_tma_mixed(const StepParams* Ps, const CUtensorMap* tin, const CUtensorMap* tout,
                           const BatchTile* work, int total, int nslots, unsigned int* counter, int wait_polls,
                           int recon, int grid, cudaStream_t st, bool launch, int* per_sm);

// the passive scalar's step (FP64, HLLC or HLLCQ): q (time level of P.in)
// -> q2, before the gas step of the same time level
int launch_scalar(const StepParams& P, const double* q, double* q2, int flux, int recon, double q_fixed,
                  cudaStream_t st);

// kernel parameters of a configuration (grid spacing, constants, boundaries)
inline void fill_step_params(StepParams& P, const ast_config& c)
{
    std::memset(&P, 0, sizeof P);
    P.N = c.N;
    P.M = c.M;
    P.x_min = c.x_min;
    P.dx = (c.x_max - c.x_min) / (c.N - 1);
    P.dy = (c.y_max) / (c.M);
    P.y_min = (c.y_max / (2.0 * c.M));
    P.krit_dx = c.cfl * P.dx;
    P.krit_dy = c.cfl * P.dy;
    P.dt_cap = c.dt_cap;
    P.p_floor = c.p_floor;
    P.gamma = c.gamma;
    P.tol = c.riemann_tol;
    P.max_iter = c.riemann_max_iter;
    P.x_minf = (float)P.x_min;
    P.dxf = (float)P.dx;
    P.y_minf = (float)P.y_min;
    P.dyf = (float)P.dy;
    P.p_floorf = (float)c.p_floor;
    P.body_lof = (float)c.body_lo;
    P.body_hif = (float)c.body_hi;
    P.body_rsplitf = (float)c.body_rsplit;
    P.body_ampf = (float)c.body_amp;
    P.gd = make_gas<double>(c.gamma, c.riemann_tol, c.riemann_max_iter);
    P.gf = make_gas<float>(c.gamma, c.riemann_tol, c.riemann_max_iter);
    P.geom = c.geom;
    P.grad_p = c.grad_p;
    P.collect_stats = c.collect_stats;
    // the FP32 form always iterates with the safeguarded Newton: the
    // reference's absolute bisection tolerance is below FP32 resolution
    P.riemann_newton = (c.riemann_newton || c.precision == AST_PREC_FP32) ? 1 : 0;
    P.guess = c.guess;
    P.mlp_gate = (float)c.mlp_gate;
    P.rec_every = 1;
    P.wait_polls = c.copy_wait_polls > 0 ? c.copy_wait_polls : tma::kWaitLimit;
    P.rec_gate = 0.0;
    for (int sd = 0; sd < 4; sd++) {
        P.bc_kind[sd] = c.bc[sd].kind;
        P.bc_val[sd][0] = c.bc[sd].rho;
        P.bc_val[sd][1] = c.bc[sd].p;
        P.bc_val[sd][2] = c.bc[sd].vz;
        P.bc_val[sd][3] = c.bc[sd].vr;
    }
    P.fixed_region = c.fixed_region;
    P.fixed_zc = c.fixed_zc;
    P.fixed_az2 = c.fixed_az * c.fixed_az;
    P.fixed_ar2 = c.fixed_ar * c.fixed_ar;
    {
        // index box of |z - zc| <= az, 0 <= r <= ar, widened by one cell
        auto clampi = [](double v) { return (int)std::fmax(-1e9, std::fmin(1e9, v)); };
        P.fixed_nlo = clampi(std::floor((c.fixed_zc - c.fixed_az - c.x_min) / P.dx) - 1.0);
        P.fixed_nhi = clampi(std::ceil((c.fixed_zc + c.fixed_az - c.x_min) / P.dx) + 1.0);
        P.fixed_mhi = clampi(std::ceil((c.fixed_ar - P.y_min) / P.dy) + 1.0);
    }
    P.region_select = c.region_select;
    P.skip_uniform = c.skip_uniform;
    {
        // columns whose face positions pass the reference's region test
        // lo < x < hi (x = x_min + n dx, plus dx/2 for the z face above the
        // cell; the product rounded separately, as the reference's FP64
        // expression is); x grows with n, so each set is one interval
        P.region_zlo = P.region_rlo = 1;
        P.region_zhi = P.region_rhi = 0;
        bool zin = false, rin = false;
        for (int n = -3; n <= c.N + 2; n++) {
            volatile double prod = (double)n * P.dx;   // no contraction into an FMA
            const double x = P.x_min + prod, xz = x + P.dx / 2.0;
            if (xz > c.region_lo && xz < c.region_hi) {
                if (!zin) P.region_zlo = n;
                P.region_zhi = n;
                zin = true;
            }
            if (x > c.region_lo && x < c.region_hi) {
                if (!rin) P.region_rlo = n;
                P.region_rhi = n;
                rin = true;
            }
        }
        // the tile's faces reach two columns beyond the grid
        if (P.region_zlo == -3) P.region_zlo = INT_MIN;
        if (P.region_zhi == c.N + 2) P.region_zhi = INT_MAX;
        if (P.region_rlo == -3) P.region_rlo = INT_MIN;
        if (P.region_rhi == c.N + 2) P.region_rhi = INT_MAX;
    }
    P.body_force = c.body_force;
    P.body_lo = c.body_lo;
    P.body_hi = c.body_hi;
    P.body_rsplit = c.body_rsplit;
    P.body_amp = c.body_amp;
    P.nsrc = nullptr;   // set by ast_set_neutral / ast_add_mk_raw
    P.nsrc_coef = (c.neutral_kn != 0.0) ? c.neutral_nh / c.neutral_kn : 0.0;
}

extern template int launch_step_r<double, kSoA>(const StepParams&, int, int, cudaStream_t, bool);
extern template int launch_step_r<float, kSoA>(const StepParams&, int, int, cudaStream_t, bool);
extern template int launch_step_r<double, kAoS>(const StepParams&, int, int, cudaStream_t, bool);


}  // namespace ast
