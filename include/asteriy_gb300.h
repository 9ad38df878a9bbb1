/*
 * asteriy_gb300.h - C ABI of the GB300-native explicit r-z finite-volume step.
 *
 * The reference (Asteriy_2d) has no library interface: its operator is the
 * step kernel
 *     Kernel_TVD(double2* s, double2* u, double2* s2, double2* u2,
 *                double* T, double* T_do, double* TT, int method)
 * (kernel.cu:2513), the first-order variants add2 (kernel.cu:1928) and
 * add_MK (kernel.cu:2293), and the scalar kernel funk_time (kernel.cu:1525)
 * that shifts the lagged time step.  Grid, gamma, CFL and boundary rules are
 * compile-time macros (Header.h:6-47) and hard-coded branches.  This header
 * turns all of that into a runtime configuration and a small set of entry
 * points with status-code returns.
 *
 * Conventions kept from the reference:
 *   - state layout at the boundary: two arrays of K = N*M pairs,
 *     s[k] = (rho, p) and u[k] = (v_z, v_r), k = m*N + n, n along z (the
 *     reference's x), m along r (the reference's y)  (kernel.cu:2515-2517);
 *   - cell centres z = x_min + n*dx with dx = (x_max - x_min)/(N-1) and
 *     r = y_min + m*dy with dy = y_max/M, y_min = dy/2   (Header.h:11-16);
 *   - lagged time step: a step uses T_do, the step size computed during the
 *     previous step; the first step uses dt_first (1e-9, kernel.cu:3322);
 *     after each step T_do <- new dt, TT += T_do, step += 1
 *     (funk_time, kernel.cu:1525-1536).
 *
 * All functions return AST_OK (0) or a negative AST_ERR_* code.
 * Pointers are host pointers unless a parameter says otherwise.
 */
#ifndef ASTERIY_GB300_H
#define ASTERIY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AST_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define AST_OK               0
#define AST_ERR_INVALID     -1  /* bad argument or configuration           */
#define AST_ERR_CUDA        -2  /* a CUDA runtime call failed               */
#define AST_ERR_NOMEM       -3  /* device or host allocation failed         */
#define AST_ERR_IO          -4  /* file could not be read or written        */
#define AST_ERR_UNSUPPORTED -5  /* valid request this build does not serve  */
#define AST_ERR_NUMERIC     -6  /* non-finite values appeared in the state  */

/* ---- device status bits (ast_stats.status) ----------------------------- */
#define AST_ST_RHO_FLOOR    0x01u /* rho' <= 0: old density kept (kernel.cu:3060-3064) */
#define AST_ST_P_FLOOR      0x02u /* p' <= 0: set to p_floor (kernel.cu:3070-3073)     */
#define AST_ST_NEWTON_CAP   0x04u /* two-shock Newton hit riemann_max_iter             */
#define AST_ST_BISECT_CAP   0x08u /* shock-rarefaction bisection hit its cap           */
#define AST_ST_NONFINITE    0x10u /* a wave speed or state became NaN/Inf              */
#define AST_ST_VACUUM       0x20u /* exact solver met the vacuum pattern               */
#define AST_ST_MLP_FALLBACK 0x40u /* learned guess rejected, PVRS guess used           */
#define AST_ST_TIMEOUT      0x80u /* a bulk copy did not arrive within the wait limit  */

/* ---- enumerations ------------------------------------------------------ */
/* HLLC is the Korolkov solver (HLLC_2d_Korolkov, Gas_Dinamic.cu:1814);
   HLLC_A the reference's second HLLC (HLLC_Aleksashov, kernel.cu:767), an
   MHD formulation it calls with zero magnetic field (add_MK method 1). */
enum ast_flux   { AST_FLUX_HLL = 0, AST_FLUX_HLLC = 1, AST_FLUX_GODUNOV = 2, AST_FLUX_HLLC_A = 3,
                  AST_FLUX_HLLCQ = 4 /* HLLCQ_Korolkov_2D (Gas_Dinamic.cu:249-353), FP64 solver only */ };
enum ast_recon  { AST_RECON_NONE = 0, AST_RECON_MINMOD = 1 };
enum ast_geom   { AST_GEOM_PLANAR = 0, AST_GEOM_AXISYM = 1 };
enum ast_prec   { AST_PREC_FP64 = 0, AST_PREC_FP32 = 1 };
enum ast_guess  { AST_GUESS_PVRS = 0, AST_GUESS_MLP = 1 };
enum ast_side   { AST_Z_LO = 0, AST_Z_HI = 1, AST_R_LO = 2, AST_R_HI = 3 };
/*
 * Boundary kinds.  Each side has two ghost layers, j = 0 next to the
 * boundary cell b0, j = 1 beyond it (the reference's first and second
 * neighbours, kernel.cu:2549-2619 and 2638-2698):
 *   REFLECT  ghost j = mirror of interior cell j, normal velocity negated
 *            (axis and wall rules, kernel.cu:2564-2569, 2609-2614, 2661-2698);
 *   OUTFLOW  ghost j = b0 (zero gradient, kernel.cu:2549-2553, 2639-2643);
 *   FIXED    ghost j = the side's (rho, p, vz, vr) (kernel.cu:2577-2580);
 *   SUCTION  ghost j = b0 with the normal velocity limited: on a low side
 *            v_n = min(v_n, limit), on a high side v_n = max(v_n, limit),
 *            limit = the side's vz (z sides) or vr (r sides)
 *            (add_MK, kernel.cu:2340-2354);
 *   NONREFLECT ghost j = b0 carried along the outgoing characteristic, the
 *            rule the reference leaves commented in add2 for its z_hi side
 *            (kernel.cu:1979-1985): with c = sqrt(gamma p/rho) and w the
 *            velocity along the outward normal, c_g = (gamma-1)/(gamma+1)
 *            (w + 2c/(gamma-1)), ghost w = c_g, rho = rho (c_g/c)^(2/(gamma-1)),
 *            p = rho_g c_g^2/gamma, tangential velocity kept.
 */
enum ast_bc_kind { AST_BC_REFLECT = 0, AST_BC_OUTFLOW = 1, AST_BC_FIXED = 2, AST_BC_SUCTION = 3,
                   AST_BC_NONREFLECT = 4 };

typedef struct ast_bc {
    int32_t kind;
    int32_t pad_;
    double rho, p, vz, vr;
} ast_bc;

/*
 * Runtime configuration.  Defaults from ast_config_default() reproduce the
 * reference macros (Header.h) where they exist.
 */
typedef struct ast_config {
    int32_t N, M;                 /* cells along z and r (Header.h:8-10)             */
    double  x_min, x_max, y_max;  /* domain (Header.h:11-13)                          */
    double  gamma;                /* ratio of specific heats, ggg (Header.h:17)       */
    double  cfl;                  /* krit (Header.h:47)                               */
    int32_t flux;                 /* enum ast_flux                                    */
    int32_t recon;                /* enum ast_recon                                   */
    int32_t geom;                 /* enum ast_geom                                    */
    int32_t precision;            /* enum ast_prec                                    */
    int32_t grad_p;               /* 1: reconstruct p too (grad_p, Header.h:31)       */
    int32_t guess;                /* enum ast_guess (exact solver's p* start)         */
    ast_bc  bc[4];                /* indexed by enum ast_side                         */
    /* cells with (z-fixed_zc)^2/fixed_az^2 + r^2/fixed_ar^2 < 1 keep their state
       (add_MK, kernel.cu:2317-2324); 0 disables                                     */
    int32_t fixed_region;
    int32_t region_select;        /* 1: high-order flux only on faces whose z
                                     position lies in (region_lo, region_hi), first-
                                     order HLL elsewhere (kernel.cu:2799-2857)        */
    double  fixed_zc, fixed_az, fixed_ar;
    double  region_lo, region_hi;
    /* body force Q2 = -amp*rho (r >= body_rsplit) / +amp*rho (r < body_rsplit)
       in v_r for body_lo < z < body_hi (kernel.cu:3039-3056); 0 disables           */
    int32_t body_force;
    int32_t riemann_max_iter;     /* cap for Newton / bisection (reference: none)     */
    double  body_lo, body_hi, body_rsplit, body_amp;
    double  dt_first;             /* T_do of the first step (kernel.cu:3322): 1e-9    */
    double  dt_cap;               /* per-cell tmin start (kernel.cu:2530): 1000       */
    double  p_floor;              /* pressure floor (kernel.cu:3072): 1e-6            */
    double  riemann_tol;          /* Newton/bisection tolerance, eps (Header.h:62)    */
    int32_t collect_stats;        /* 1: count Riemann iterations in ast_stats         */
    /* p* iteration of the exact solver: 0 = the reference's (bisection for
       shock-rarefaction, Newton from the acoustic value for two shocks,
       kernel.cu:220-231); 1 = safeguarded Newton on the full pressure
       function for both patterns, started from `guess`.  The FP32 form
       always uses 1 (the reference's absolute tolerance is below FP32
       resolution).                                                          */
    int32_t riemann_newton;
    /* the FP32 solver's step kernel: 2 = strips of 30 columns swept up
       their rows by one warp each, the stencil, fluxes and update in
       registers (the learned start value by the whole warp, in FP32);
       1 = the persistent tile kernel (tiles staged and stored by
       bulk-tensor copies, double-buffered; the learned start value by f16
       tensor-core tiles); 0 = one CTA per tile.  The same arithmetic per
       face and cell.  The FP64 solver with 1 runs the persistent tile
       kernel for the HLL family on grids of at least two 32x16 tiles per
       SM, one CTA per tile otherwise (the exact solver: one CTA per tile);
       the raw entry points always use one CTA per tile (default 1)         */
    int32_t persistent;
    /* 1: tiles whose staged cells (tile and two-cell halo, ghosts included)
       all hold the same four values, bit for bit, skip the face pass: every
       face of such a tile has the same flux, so the flux differences of the
       update are exactly zero, and the update runs on zero fluxes; the wave
       speeds come from one face of each orientation.  The results are
       identical to the full computation.  Tiles near the fixed region, runs
       with region_select, and uniform states whose flux is not finite take
       the full path.  With HLL in the FP32 form it also lets face pairs whose
       five stencil cells are one state in a whole warp skip the
       reconstruction (the same results; faster where the gas is undisturbed,
       some per cent slower where every face is disturbed) (default 0)      */
    int32_t skip_uniform;
    /* polls of a bulk tile copy's barrier before the FP32 persistent kernels
       report AST_ST_TIMEOUT (the copy is then waited for with the long
       default limit and the tile computed, so the step's result is the
       same; ast_synchronize returns AST_ERR_CUDA).  0: the default, about a
       second; small values make the failure path run (tests)            */
    int32_t copy_wait_polls;
    int32_t reserved_i[3];
    /* wave strength above which the learned start value is used:
       max(|ln(p_R/p_L)|, |u_R - u_L| / min(c_L, c_R)); weaker faces start
       from the acoustic value, which is already close for them (0.2)        */
    double  mlp_gate;
    /* characteristic inflow at z_lo after every step (add2_bound,
       kernel.cu:1895-1925; p_H = inflow_p, inflow speed inflow_v): cell
       column n = 0 becomes rho = pp/(gamma-1)/T0, p = inflow_p,
       (v_z, v_r) = (inflow_v, 0), with T0 = inflow_p/(gamma-1) and
       pp = p'(1) - rho(0) c(0) (v_z'(1) - inflow_v), primes the new state of
       column 1, unprimed the old state of column 0.  0 disables (default);
       the reference's values are 7 and 1.                                  */
    double  inflow_p, inflow_v;
    /* neutral-atom coupling (add_MK, kernel.cu:2495-2496): with a source
       array set (ast_set_neutral, ast_add_mk_raw) the momentum gains
       T_do * (rho * neutral_nh / neutral_kn) * (nn2.x, nn2.y) per step;
       the reference's n_H and Kn (Header.h:84-85) are the defaults, 3 and
       0.419231 (neutral_kn = 0: no source).  The energy term of add_MK
       multiplies its source by 0 and is left out.                           */
    double  neutral_nh, neutral_kn;
    /* the passive scalar's value in the ghost cells of FIXED sides
       (ast_set_scalar; other sides copy or mirror the scalar as the
       state's ghost rules do) */
    double  scalar_in;
    double  reserved_d[2];
} ast_config;

typedef struct ast_stats {
    uint32_t status;              /* OR of AST_ST_* bits since the last reset         */
    uint32_t newton_max_iters;    /* largest iteration count of one Newton solve      */
    uint64_t rho_floor;           /* cells that hit the density floor                 */
    uint64_t p_floor;             /* cells that hit the pressure floor                */
    uint64_t newton_calls, newton_iters;
    uint64_t bisect_calls, bisect_iters;
    uint64_t mlp_fallback;        /* learned guesses replaced by the PVRS guess       */
    uint64_t strong_calls;        /* iterative faces above mlp_gate (both start values) */
    uint64_t strong_iters;        /* their Newton iterations                          */
    uint64_t reserved[2];
} ast_stats;

typedef struct ast_solver ast_solver;

/* Learned start value of the exact solver: parameter block of the 6-32-32-1
   SiLU network (feature shift[6], scale[6], W1[32][6], b1[32], W2[32][32],
   b2[32], w3[32], b3). */
#define AST_MLP_NPARAM 1325
/* One recorded face of the exact solver (training data of the network):
   features x[6], target log(p* / p_L), then step, face id and wave pattern
   stored as int32 bit patterns. */
#define AST_RECORD_FLOATS 10

/* ---- library ----------------------------------------------------------- */
int         ast_abi_version(void);
const char* ast_strerror(int code);
/* Text of the last failure on the calling thread ("" if none). */
const char* ast_last_error(void);
/* sizeof(ast_config) and sizeof(ast_stats) as compiled into the library,
   for bindings that mirror the structures. */
size_t      ast_sizeof_config(void);
size_t      ast_sizeof_stats(void);
/* Fills *cfg with the reference's macro values: gamma 5/3, CFL 0.05,
   HLL + minmod, planar, FP64, reflect on r sides, outflow on z sides,
   dt_first 1e-9, dt_cap 1000, p_floor 1e-6, riemann_tol 1e-9. */
void        ast_config_default(ast_config* cfg);
int         ast_config_check(const ast_config* cfg);

/* ---- solver object (replaces main's allocation + time loop,
        kernel.cu:3283-3298 and 3868-3947) ------------------------------- */
int ast_create(const ast_config* cfg, ast_solver** out);
int ast_destroy(ast_solver* solver);
/* Runs on the given cudaStream_t (NULL = the legacy default stream). */
int ast_set_stream(ast_solver* solver, void* cuda_stream);
/* s, u: K (rho,p) and K (v_z,v_r) pairs; on_device=1 means device pointers. */
int ast_set_state(ast_solver* solver, const double* s, const double* u, int on_device);
int ast_get_state(ast_solver* solver, double* s, double* u, int on_device);
int ast_set_clock(ast_solver* solver, double T_do, double TT, int64_t step);
int ast_get_clock(ast_solver* solver, double* T_do, double* TT, int64_t* step);
/* Enqueues nsteps steps (ping-pong, lagged dt) on the solver's stream and
   returns without waiting; ast_synchronize waits and reports errors. */
int ast_step(ast_solver* solver, int nsteps);
int ast_synchronize(ast_solver* solver);
/* One step from host arrays to host arrays, waiting for the result: the
   reference's step between its host<->device state copies (the state
   in, kernel.cu:3444-3445; the time loop, 3868-3947; the state out,
   4075-4076).
   s_in, u_in hold the state in the layout of ast_set_state; s_out, u_out
   receive the new state in the layout of ast_get_state.  An output array
   may be its input array (in place); any other overlap is AST_ERR_INVALID.
   Page-locked arrays are moved in bands of rows, the copies in, the step
   and the copies out overlapping; pageable arrays, a configuration with
   the inflow rule, or the FP32 form with a neutral-coupling source take
   ast_set_state + ast_step + ast_get_state. */
int ast_step_host(ast_solver* solver, const double* s_in, const double* u_in, double* s_out, double* u_out);
/* nsteps such steps between two pairs of host arrays: step k reads
   (s_a, u_a) and writes (s_b, u_b) for even k, the reverse for odd k, so
   the result is in (s_b, u_b) when nsteps is odd and in (s_a, u_a) when it
   is even.  Every step copies its whole input in and its whole result
   out; with page-locked arrays a band of step k + 1 goes in as soon as the
   same band of step k is out, so the copies of consecutive steps overlap.
   Same array rules and fallbacks as ast_step_host; the pairs may be the
   same arrays (in place). */
int ast_step_host_n(ast_solver* solver, int nsteps, double* s_a, double* u_a, double* s_b, double* u_b);
/* The neutral-coupling momentum source of add_MK (kernel.cu:2495-2496):
   nn2 holds K (x, y, z) triples in the reference's double3 layout (only x
   and y enter the update); on_device=1 means a device pointer.  The solver
   keeps its own copy; nn2 = NULL removes the source.  See
   ast_config.neutral_nh.  The FP64 solver adds the source inside the
   update, as add_MK does; the FP32 form adds it in a pass after the step
   (same terms, in FP64, at the step's total energy). */
int ast_set_neutral(ast_solver* solver, const double* nn2, int on_device);
int ast_get_stats(ast_solver* solver, ast_stats* out, int reset);
/* ---- passive scalar (FP64 solver; flux AST_FLUX_HLLC or AST_FLUX_HLLCQ;
   no region_select).  The reference's HLLC solvers compute a passive
   scalar's face flux beside the gas flux (the Q channel of
   HLLC_2d_Korolkov_b_s, Gas_Dinamic.cu:1660-1808; HLLCQ_Korolkov_2D,
   Gas_Dinamic.cu:249-353) but its steps never carry one.  With a scalar set,
   every ast_step also advances Q, a density carried by the flow: from the
   same old state, with the same reconstruction (the density's rule) and
   solver as the gas step, Q' = Q - T_do/(dx dy) * (sum of its face fluxes)
   [- T_do/r * Q * v_r on the axisymmetric grid]; cells held fixed keep Q;
   ghost values as the state's (FIXED sides: cfg.scalar_in).  The gas step
   is unchanged.  q holds K = N*M values, index m*N + n; on_device = 1
   means a device pointer.  q = NULL removes the scalar.  The host-array
   steps (ast_step_host*) refuse a solver that carries one. */
int ast_set_scalar(ast_solver* solver, const double* q, int on_device);
int ast_get_scalar(ast_solver* solver, double* q, int on_device);
/* Profiling builds only (the library compiled with AST_PHASE_CLOCKS;
   otherwise AST_ERR_UNSUPPORTED): SM cycles the FP32 persistent kernel's
   CTAs spent per phase of their tiles since the last reset, summed over
   CTAs: out[0] tile arrival (the barrier after a tile's bulk copy
   arrives), [1] ghost cells, [2] face pass, [3] exact-solver queue, [4]
   update, [5] final store and report, [6] CTAs, [7] tiles.  reset = 1
   zeroes the counters after reading. */
int ast_get_phase_clocks(ast_solver* solver, uint64_t out[8], int reset);
/* Device view of the current state: four planes rho, p, v_z, v_r of M rows
   with row pitch *ld elements of *elem_bytes bytes (8 = FP64, 4 = FP32),
   plane stride ld*M.  Valid until the next ast_step / ast_set_state. */
int ast_device_state(ast_solver* solver, void** planes, int64_t* ld, int* elem_bytes);

/* ---- learned start value of the exact solver (no reference counterpart:
        the reference always starts from the acoustic value, kernel.cu:641-642)
   A solver created with guess == AST_GUESS_MLP and riemann_newton == 1 (or
   FP32 precision) starts every iterative p* solve from the network's
   prediction p_L exp(y) and falls back to the acoustic start value when the
   prediction lies outside the pattern's bracket (counted in mlp_fallback).
   The call copies the parameters to the device, writes beside them the
   network's packed form that the step kernels copy into shared memory, and
   waits for the solver's stream.                                          */
int ast_set_mlp(ast_solver* solver, const float* params);  /* AST_MLP_NPARAM host floats */
/* Watch cells: the density of the current state at n cells (indices
   k = m*N + n into the state) and the solver's time TT, the reference's
   probe kernel funk_my (kernel.cu:1538-1545) that its loop samples every
   200 steps into "TT rho" series (kernel.cu:3547-3555, 3950-3960).
   Waits for the solver's stream. */
int ast_probe(ast_solver* solver, const int64_t* cells, int n, double* rho, double* TT);
/* Face recorder: on the following steps with step % every == 0, every exact-
   solver face that needs the iterative p* solve and whose wave strength
   max(|ln(p_R/p_L)|, |u_R-u_L|/min(c_L,c_R)) exceeds min_strength (0 keeps
   all) is written as one record of AST_RECORD_FLOATS floats, up to
   `capacity` records (device buffer owned by the solver).  ast_record_stop
   returns the number of faces offered, which may exceed the capacity;
   ast_record_read copies min(n, stored) records.  FP64 exact-Godunov
   solvers only (the records are training targets of the learned start
   value); other solvers return AST_ERR_UNSUPPORTED. */
int ast_record_start(ast_solver* solver, int64_t capacity, int every, double min_strength);
int ast_record_stop(ast_solver* solver, int64_t* offered);
int ast_record_read(ast_solver* solver, float* out, int64_t n);
/* Training kernels (host arrays in and out, work on the current device).
   samples: n records as written by the recorder (x[6], target, ...). */
int ast_mlp_init(const float* samples, int64_t n, uint64_t seed, float* params);
int ast_mlp_grad(const float* params, const float* samples, int64_t n, float* grad, float* loss);
int ast_mlp_forward(const float* params, const float* x, int64_t n, int stride, float* y);
/* The step kernel's inference path (f16 tensor-core tiles of 16 faces) on
   given feature rows, to compare it with the FP32 network above. */
int ast_mlp_forward_tc(const float* params, const float* x, int64_t n, int stride, float* y);
int ast_mlp_train(const float* samples, int64_t n, int epochs, int batch, float lr, uint64_t seed,
                  float* params, float* loss_per_epoch);

/* ---- kernel-level drop-in ----------------------------------------------
 * One step on reference-layout device arrays, the replacement for
 *   Kernel_TVD<<<K/256,256>>>(s, u, s2, u2, T, T_do, TT, method)
 * (kernel.cu:2513, launched at kernel.cu:3874).  Reads s, u and *T_do,
 * writes s2, u2 and lowers *T to min(*T, new dt) exactly (the reference's
 * racy write, kernel.cu:3013-3017, becomes an atomic min).  method is kept
 * for signature compatibility and ignored: cfg->flux selects the flux.
 * All pointers are device pointers; cuda_stream may be NULL.
 */
int ast_step_raw(const double* s, const double* u, double* s2, double* u2,
                 double* T, const double* T_do, const double* TT, int method,
                 const ast_config* cfg, void* cuda_stream);
/* The same for
     add_MK<<<K/256,256>>>(s, u, s2, u2, nn1, nn2, nn3, T, T_do, method, step)
   (kernel.cu:2293, launched at kernel.cu:3723 and 3747), with its
   neutral-coupling momentum source from nn2 (K double3, device pointer;
   NULL: none).  nn1 and nn3 are accepted and not read (add_MK reads nn1
   nowhere and multiplies its nn3 term by 0); method and step are ignored
   like ast_step_raw's method.  cfg->geom should be AST_GEOM_AXISYM for
   add_MK's update. */
int ast_add_mk_raw(const double* s, const double* u, double* s2, double* u2, const double* nn1,
                   const double* nn2, const double* nn3, double* T, const double* T_do, int method, int step,
                   const ast_config* cfg, void* cuda_stream);
/* The same for the first-order planar step
     add2<<<K/256,256>>>(s, u, s2, u2, T, T_do, TT, method, step)
   (kernel.cu:1928-2291, launched at kernel.cu:3488, 3512, 3564, 3589),
   reproduced as the reference evaluates it: each cell its own four faces,
   HLLC on its right and r faces inside the region (region_lo, region_hi)
   and HLL outside, and on its LEFT face HLL inside the region and HLLC
   outside (kernel.cu:2078-2085: the two cells of one face use different
   fluxes there); right side outflow, left side the z_lo FIXED state with
   its density perturbed by 1 + 0.01 sin(2 pi *TT) for y < 0.5 while
   *TT < 3 when method != 0; reflecting r sides; the body force of
   ast_config (the reference's is 2.5 rho for 20 < z < 30).  Lowers *T to
   the cells' smallest dt candidate (atomic).  cfg must be FP64, first
   order (recon NONE), planar, with a FIXED z_lo side; region_select 0
   means no region (HLL right and r faces, HLLC left faces).  step is
   ignored.  Device pointers. */
int ast_add2_raw(const double* s, const double* u, double* s2, double* u2, double* T, const double* T_do,
                 const double* TT, int method, int step, const ast_config* cfg, void* cuda_stream);
/* Replacement for add2_bound<<<K/256,256>>>(s, u, s2, u2, ...)
   (kernel.cu:1895-1925, launched after the step at kernel.cu:3565, 3590):
   column n = 0 of (s2, u2) from the old state (s, u) and the new column 1,
   as described at ast_config.inflow_p (which must be positive; the
   reference's p_H is 7, its inflow speed 1).  Device pointers. */
int ast_inflow_raw(const double* s, const double* u, double* s2, double* u2, const ast_config* cfg,
                   void* cuda_stream);
/* Replacement for funk_time<<<1,1>>>(T, T_do, TT, i) (kernel.cu:1525-1536):
   T_do = T; TT += T_do; T = 1e7; i += 1.  Device pointers. */
int ast_funk_time(double* T, double* T_do, double* TT, int* i, void* cuda_stream);

/* ---- a step that allocates nothing (no counterpart in the reference) -----
 * For callers that must not call cudaMalloc while they step: a process whose
 * device memory is handed out by a different allocator under a fixed
 * budget, or a real-time loop that cannot absorb an allocation's latency or
 * failure.  It does what ast_step_raw + ast_funk_time do: reads s, u and
 * *T_do, writes s2, u2, then *T_do = the new dt, *TT += *T_do, *step += 1
 * (and *status = the step's AST_ST_* bits when status is not NULL).  It
 * enqueues three kernels on cuda_stream: a one-thread copy of T_do, TT and
 * step into the scratch array below, the step kernel, and a one-thread copy
 * back out.  All pointers are device pointers, FP64 reference layout; guess
 * must be PVRS.  Its cross-CTA reduction state lives in a file-scope device
 * array of AST_NOALLOC_SCRATCH_BYTES per device, held from library load to
 * process exit; it does not grow with the grid.  Every call shares that
 * array and clears all of it first, so calls that overlap on the GPU (other
 * streams or host threads) race and must be serialised by the caller.  The
 * first call on a device looks the array up and sets kernel attributes:
 * make it before any stream capture. */
#define AST_NOALLOC_SCRATCH_BYTES 256
int ast_step_noalloc(const double* s, const double* u, double* s2, double* u2, double* T_do, double* TT,
                     int64_t* step, unsigned int* status, const ast_config* cfg, void* cuda_stream);

/* ---- batched problems (no counterpart in the reference, which runs one
        problem per process) ---------------------------------------------
 * A batch holds nprob independent problems of one precision, each with its
 * own grid, gas, flux, reconstruction, geometry, boundaries, clock and
 * lagged dt.  ast_batch_step advances every problem by nsteps steps of its
 * own dt.  A step is one kernel launch per (flux, recon) class present,
 * each over a work list of (problem, tile) pairs, the problems' tiles
 * concatenated.  Steps are captured in blocks of 16 into a CUDA graph in
 * which every class is its own chain of launches (the classes' problems are
 * independent), forked from the batch's stream and joined back at the end
 * of the block.  Problem states live in one device arena.  guess == MLP
 * problems share the network given to ast_batch_set_mlp. */
typedef struct ast_batch ast_batch;
#define AST_BATCH_MAX 4096
int ast_batch_create(const ast_config* cfgs, int nprob, ast_batch** out);
int ast_batch_destroy(ast_batch* batch);
int ast_batch_set_stream(ast_batch* batch, void* cuda_stream);
/* state of problem `prob` in the layout of ast_set_state / ast_get_state */
int ast_batch_set_state(ast_batch* batch, int prob, const double* s, const double* u, int on_device);
int ast_batch_get_state(ast_batch* batch, int prob, double* s, double* u, int on_device);
int ast_batch_set_clock(ast_batch* batch, int prob, double T_do, double TT, int64_t step);
int ast_batch_get_clock(ast_batch* batch, int prob, double* T_do, double* TT, int64_t* step);
int ast_batch_step(ast_batch* batch, int nsteps);
/* waits for the batch's stream; AST_ERR_NUMERIC if any problem's state
   became non-finite */
int ast_batch_synchronize(ast_batch* batch);
int ast_batch_get_stats(ast_batch* batch, int prob, ast_stats* out, int reset);
int ast_batch_set_mlp(ast_batch* batch, const float* params);
/* cells of all problems, tiles of all problems (at the tile shapes in use),
   and kernel launches per step (the number of (flux, recon) classes, or 1
   in the one-launch mode) */
int ast_batch_info(ast_batch* batch, int64_t* cells, int64_t* tiles, int* launches_per_step);
/* the number of (flux, recon) classes */
int ast_batch_num_classes(ast_batch* batch);
/* Schedules.  Each class steps with one schedule: 0, 1, 2 = one CTA per
 * tile with tiles of 32x16, 16x16 or 64x8 (z x r) cells; 3 = the persistent
 * batch kernel (FP32 only; the class's tiles of 32x16 staged and stored by
 * bulk-tensor copies, the default for FP32 batches; FP64 batches default to
 * 0; the last CTA of each launch shifts every problem's dt); 4 = the
 * single-problem persistent kernel once per problem, each
 * problem its own chain of launches in the step graph (FP32 only).
 * ast_batch_autotune times every schedule on every class, `trials` steps
 * each on the current state (each trial reads the current time level and
 * writes the other; the clocks and counters are restored afterwards, so the
 * run continues exactly as without the call) and keeps the fastest per
 * class.  ast_batch_class reports class `cls` (0 <= cls < launches_per_step):
 * its flux, reconstruction, problem count, schedule and tile shape in use,
 * and the tuner's ms per step of each schedule (AST_BATCH_SCHEDULES floats,
 * 0 when not timed or not built); ast_batch_set_schedule and
 * ast_batch_set_tiles (one CTA per tile, the given shape) set a class's
 * schedule by hand. */
#define AST_BATCH_SCHEDULES 5
int ast_batch_autotune(ast_batch* batch, int trials);
int ast_batch_class(ast_batch* batch, int cls, int* flux, int* recon, int* nprob, int* schedule, int* tile_z,
                    int* tile_r, float* ms_per_schedule);
int ast_batch_set_schedule(ast_batch* batch, int cls, int schedule);
int ast_batch_set_tiles(ast_batch* batch, int cls, int tile_z, int tile_r);
/* One launch per step for the whole batch (FP32 batches whose problems
 * share one reconstruction): every problem's 32x16 tiles in one work list
 * (slot order: the exact solver's problems first, larger problems first),
 * each tile stepped with the tile code of its problem's flux, instead of
 * one launch per class.  on = 1: a CTA per tile; on = 2: the persistent
 * kernel (as many CTAs as fit take tiles from one counter, each tile staged
 * by a bulk-tensor copy through its problem's tensor map while the previous
 * tile computes); 0: one launch per class.  The results are those of
 * schedule 0 for every class, bit for bit.  ast_batch_autotune, after the
 * per-class schedules, times a whole step all three ways and keeps the
 * fastest; ast_batch_get_mixed reports the mode in use, the faster
 * one-launch mode's time and the per-class launches' (ms per step, 0 when
 * not timed).  ast_batch_set_mixed(batch, 1 or 2) on a batch that cannot
 * run this way is AST_ERR_UNSUPPORTED. */
int ast_batch_set_mixed(ast_batch* batch, int on);
int ast_batch_get_mixed(ast_batch* batch, int* on, float* ms_mixed, float* ms_split);

/* A seeded set of benchmark problems: problem i draws, in this order from
 * one std::mt19937_64(seed) stream (u = (draw >> 11) * 2^-53, b = draw >> 63):
 *   size   M = round(64 * 8^u), N = 2M           (128x64 .. 1024x512)
 *   mach   1.5 + 4.5 u
 *   gamma  5/3 if b == 0, else 1.4
 *   setup  blast if b == 0, else wind
 *   flux   HLLC if b == 0, else exact Godunov
 *   seed   one draw (the wind setup's density-noise seed)
 * Blast: the blast problem of the single-problem benchmarks with the
 * driver pressure of a normal shock of that Mach number into the ambient
 * gas, p_in = p_out (2 gamma mach^2 - (gamma-1))/(gamma+1), p_out = 0.1.
 * Wind: the wind-counterflow problem with counterflow Mach `mach`
 * (rho = 1, p = 1/gamma, v_z = -mach).  Both: minmod, axisymmetric,
 * CFL 0.4, the given precision. */
enum ast_setup { AST_SETUP_BLAST = 0, AST_SETUP_WIND = 1 };
typedef struct {
    ast_config cfg;
    int setup;              /* enum ast_setup */
    int reserved_i;
    double mach;
    uint64_t seed;
    double reserved_d[5];
} ast_problem;
int ast_problem_set(uint64_t seed, int nprob, int precision, ast_problem* out);
/* initial state of a drawn problem (K = N*M pairs each) */
int ast_problem_fill(const ast_problem* prob, double* s, double* u);

/* ---- problem set-up and files (host) ------------------------------------ */
/* Axisymmetric blast: rho=1, v=0, p=p_in for z^2+r^2 < radius^2, else p_out. */
int ast_fill_blast(const ast_config* cfg, double p_in, double p_out, double radius,
                   double* s, double* u);
/* Wind-counterflow: counterflow (rho_inf, p_inf, v_inf along z) with uniform
   density noise in [-noise, noise] (one std::mt19937_64 draw per cell in k
   order, u = (draw >> 11) * 2^-53, factor 1 + noise*(2u-1)); inside the wind
   sphere R < r_w: rho = rho_w (r_w/R)^2, radial speed v_w,
   p = rho_w v_w^2/(gamma mach_w^2) (r_w/R)^(2 gamma). */
int ast_fill_wind(const ast_config* cfg, double r_w, double rho_w, double v_w, double mach_w,
                  double rho_inf, double p_inf, double v_inf, double noise, uint64_t seed,
                  double* s, double* u);
/* 6 doubles per cell (x, y, rho, p, vx, vy), k order (kernel.cu:4111-4148;
   read side kernel.cu:3414-3436). */
int ast_write_bin(const ast_config* cfg, const double* s, const double* u, const char* path);
int ast_read_bin(const ast_config* cfg, double* s, double* u, const char* path);
/* Tecplot FEPOINT quadrilateral file, every stride-th cell, variables
   X Y Ro P Vx Vy Mach omega (print_file_mini, kernel.cu:3109-3173). */
int ast_write_tecplot(const ast_config* cfg, const double* s, const double* u,
                      int stride, double soltime, const char* path);
/* The end-of-run Tecplot file ("_param_for_texplot_mini.txt",
   kernel.cu:4125-4129, 4156-4215): every stride-th cell, variables
   X Y Ro P Vx Vy Mach T Zav with T = p/rho and the vorticity
   Zav = dvr/dz - dvz/dr by central differences (0 on the outer cells). */
int ast_write_tecplot_final(const ast_config* cfg, const double* s, const double* u, int stride,
                            const char* path);
/* The axis line ("_param_y=0.txt", kernel.cu:4151-4164): the cells of the
   first row, one line each: x y rho p vx vy 1/c (0 where rho <= 0). */
int ast_write_axis(const ast_config* cfg, const double* s, const double* u, const char* path);
/* The run summary ("_inform.txt", kernel.cu:4166-4169): time, grid, domain
   and the problem's Mach number and chi. */
int ast_write_inform(const ast_config* cfg, double TT, double mach_inf, double chi, const char* path);

#ifdef __cplusplus
}
#endif
#endif /* ASTERIY_GB300_H */
