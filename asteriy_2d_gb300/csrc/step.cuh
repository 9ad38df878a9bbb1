// step.cuh - the fused explicit r-z step: one kernel per time step.
//
// A CTA owns a TZ x TR tile of cells.  It stages the tile plus a two-cell
// halo of (rho, p, v_z, v_r) in shared memory, filling halo cells outside
// the domain with the side's ghost rule; evaluates every z face and every r
// face of the tile once (minmod reconstruction + the configured flux);
// updates each cell from its four faces with the planar (Kernel_TVD,
// kernel.cu:3027-3073) or axisymmetric (add_MK, kernel.cu:2480-2509)
// conservative update; and reduces the largest wave speed per direction.
// The last CTA to finish turns the two maxima into the next dt and performs
// the reference's funk_time shift (kernel.cu:1525-1536) on the device, so a
// sequence of steps needs no host round trip.
//
// Exact-Godunov faces are processed in two phases: every face is classified
// (godunov_pre) and the closed-form patterns are finished at once, while the
// faces that need an iterative p* solve are pushed to a shared-memory queue
// and solved afterwards by all threads of the CTA, so that the iterations
// run in full warps instead of in one or two lanes of many warps.
#pragma once

#include <cstddef>
#include <type_traits>

#include "mlp.cuh"
#include "physics.cuh"
#include "tma.cuh"

namespace ast {

constexpr int kThreads = 256;
// the thread of the persistent kernels that issues the bulk copies: lane 0
// of the last warp (in the face pass the first two warps take one face more
// than the others)
constexpr int kCopyThread = kThreads - 32;
// the persistent kernels' tile, z x r cells: their shared-memory buffers are
// the boxes of the tensor maps the host encodes (TZ + 8 x TR + 4 cells
// loaded, TZ x TR stored), so every encoder of those maps takes these
constexpr int kTmaTZ = 32, kTmaTR = 16;

// device-resident clock and counters of a solver (one per solver)
struct DevClock {
    double T_do;                   // dt the next step uses
    double TT;                     // accumulated time
    long long step;                // steps taken
    unsigned long long smax_z;     // bits of the largest z-face wave speed (>= 0)
    unsigned long long smax_r;     // same for r faces
    unsigned int done;             // CTAs of the current step that finished
    unsigned int status;           // OR of AST_ST_* bits
    unsigned long long cnt[10];    // rho_floor, p_floor, newton_calls, newton_iters,
                                   // bisect_calls, bisect_iters, mlp_fallback, newton_max,
                                   // strong_calls, strong_iters
    unsigned int next_tile;        // persistent kernel: next tile to hand out
    unsigned int pad_;
    double T_prev;                 // dt the last step used
    unsigned long long phase[8];   // builds with AST_PHASE_CLOCKS: SM cycles per phase (phase_mark)
};

// ------------------------------------------------------------------ phase clocks
// Builds with AST_PHASE_CLOCKS only (a profiling build; otherwise every
// mark is empty): thread 0 of each CTA of the persistent kernels adds the
// SM cycles between consecutive marks to one counter per phase, and at the
// CTA's end adds them to its problem's clock.  Each mark follows the
// CTA-wide barrier that ends its phase, so a phase's cycles include the
// wait for the CTA's slowest warp.  Phases: 0 tile arrival (the barrier
// after the copy's arrival: the previous tile's slowest update and any copy
// wait), 1 ghost cells, 2 face pass, 3 exact-solver queue, 4 update (thread
// 0's own cells), 5 the final store and report; counters 6 and 7 count the
// CTAs and the tiles.
constexpr int kPhaseStart = -1, kPhaseFlush = -2;
#ifdef AST_PHASE_CLOCKS
__device__ __forceinline__ void phase_mark(int k, DevClock* C = nullptr)
{
    __shared__ long long s_t;
    __shared__ unsigned long long s_acc[8];
    if (threadIdx.x != 0) return;
    const long long now = clock64();
    if (k == kPhaseStart) {
        for (int i = 0; i < 8; i++) s_acc[i] = 0ull;
    } else if (k == kPhaseFlush) {
        if (C != nullptr) {
            s_acc[6] = 1ull;
            for (int i = 0; i < 8; i++) atomicAdd(&C->phase[i], s_acc[i]);
        }
    } else {
        s_acc[k] += (unsigned long long)(now - s_t);
        if (k == 0) s_acc[7] += 1ull;
    }
    s_t = now;
}
#else
__device__ __forceinline__ void phase_mark(int, DevClock* = nullptr) {}
#endif

enum Layout { kSoA = 0, kAoS = 1 };

struct __align__(16) StepParams {
    int N, M;
    long long ld;                  // SoA row pitch in elements
    long long plane;               // SoA plane size in elements
    double x_min, dx, y_min, dy;
    double krit_dx, krit_dy;       // cfl*dx and cfl*dy
    double dt_cap, p_floor;
    double gamma, tol;
    int max_iter;
    int geom, grad_p, collect_stats;
    int riemann_newton, guess;     // exact solver: p* iteration and its start value
    float mlp_gate;                // wave strength above which the learned start is used
    int bc_kind[4];
    double bc_val[4][4];           // rho, p, vz, vr of FIXED sides; vz/vr limit of SUCTION
    int fixed_region;
    double fixed_zc, fixed_az2, fixed_ar2;
    int fixed_nlo, fixed_nhi, fixed_mhi;   // cells that can lie in the region (one cell of margin)
    int region_select;
    int skip_uniform;              // uniform tiles skip the face pass
    // one step launched in bands of tile rows: this launch steps tile rows
    // [band_lo, band_hi) (band_hi 0: all rows of the grid), and `units` CTAs
    // of all the step's launches report to the clock (0: this launch's grid)
    int band_lo, band_hi, units;
    // polls of a bulk copy's mbarrier before a persistent kernel reports
    // AST_ST_TIMEOUT (it then waits on with the long default limit)
    int wait_polls;
    // the high-order region as column intervals (found on the host from
    // the reference's FP64 face positions): z faces whose lower cell's
    // column lies in [region_zlo, region_zhi], r faces of the columns in
    // [region_rlo, region_rhi]
    int region_zlo, region_zhi, region_rlo, region_rhi;
    int body_force;
    double body_lo, body_hi, body_rsplit, body_amp;
    // the neutral-coupling momentum source of add_MK: null, or per cell
    // (nn2.x, nn2.y) as two SoA planes of the state's precision and pitch
    // (solver) or the reference's double3 array (raw entry points); the
    // momentum gains T_do * (rho * nsrc_coef) * (nn2.x, nn2.y)
    const void* nsrc;
    double nsrc_coef;
    // state: SoA planes (in/out) or reference AoS (s, u, s2, u2)
    const void* in;
    void* out;
    const double* in_u;
    double* out_u;
    DevClock* clock;               // solver mode
    double* T_min;                 // raw mode: *T_min = min(*T_min, dt), atomic
    const double* T_do_ptr;        // raw mode: the step's dt
    unsigned int* status_ptr;      // raw mode: status bits (may be null)
    const float* mlp;              // AST_MLP_NPARAM floats (guess == MLP)
    Gas<double> gd;                // gas constants, precomputed on the host
    Gas<float> gf;
    // FP32 copies of the grid and source constants (conversions between
    // double and float run on the FP64 pipe, 1/64 of the FP32 rate)
    float x_minf, dxf, y_minf, dyf, p_floorf, body_lof, body_hif, body_rsplitf, body_ampf;
    float* rec;                    // face recorder: AST_RECORD_FLOATS per record, or null
    unsigned long long* rec_n;     // records written (may exceed rec_cap)
    long long rec_cap;
    int rec_every;                 // record on steps with step % rec_every == 0
    double rec_gate;               // record faces with wave strength above this
};

// the gas constants of the arithmetic R
template <typename R>
__device__ __forceinline__ const Gas<R>& gas_of(const StepParams& P)
{
    return *reinterpret_cast<const Gas<R>*>(sizeof(R) == 8 ? (const void*)&P.gd : (const void*)&P.gf);
}

// the NONREFLECT ghost state from the boundary cell's state v (rho, p, vz,
// vr): carried along the outgoing characteristic (the rule the reference
// leaves commented in add2, kernel.cu:1979-1985, written there for the z_hi
// side; w is the velocity along the side's outward normal)
template <typename R>
__device__ __forceinline__ void ghost_nonreflect_s(const Gas<R>& g, bool low, R& rho, R& p, R& vn)
{
    const R w = low ? -vn : vn;
    const R cc = sqrt(g.ga * p / rho);
    const R cg = g.g1 / g.g2 * (w + R(2) / g.g1 * cc);
    rho = rho * pow(cg / cc, R(2) / g.g1);
    p = rho * cg * cg / g.ga;
    vn = low ? -cg : cg;
}
// (the element chosen by branches, not by a reference to a runtime-chosen
// element, which would put the array in local memory)
template <typename R>
__device__ __forceinline__ void ghost_nonreflect(const Gas<R>& g, bool zside, bool low, R v[4])
{
    if (zside) ghost_nonreflect_s(g, low, v[0], v[1], v[2]);
    else ghost_nonreflect_s(g, low, v[0], v[1], v[3]);
}

// the SUCTION rule on v's normal velocity: on a low side v_n = min(v_n,
// lim), on a high side v_n = max(v_n, lim)
template <typename R>
__device__ __forceinline__ void ghost_suction(bool zside, bool low, R lim, R v[4])
{
    if (zside) {
        if (low) { if (v[2] > lim) v[2] = lim; }
        else     { if (v[2] < lim) v[2] = lim; }
    } else {
        if (low) { if (v[3] > lim) v[3] = lim; }
        else     { if (v[3] < lim) v[3] = lim; }
    }
}

// ------------------------------------------------------------------ loads
template <typename R, int LAYOUT>
__device__ __forceinline__ void read_cell(const StepParams& P, int n, int m, R v[4])
{
    if (LAYOUT == kSoA) {
        const R* q = (const R*)P.in;
        long long k = (long long)m * P.ld + n;
        v[0] = q[k];
        v[1] = q[k + P.plane];
        v[2] = q[k + 2 * P.plane];
        v[3] = q[k + 3 * P.plane];
    } else {
        long long k = (long long)m * P.N + n;
        double2 s = ((const double2*)P.in)[k];
        double2 u = ((const double2*)P.in_u)[k];
        v[0] = (R)s.x; v[1] = (R)s.y; v[2] = (R)u.x; v[3] = (R)u.y;
    }
}

// state of cell (n, m); a cell outside the domain follows the ghost rule of
// the side it lies beyond (include/asteriy_gb300.h).  Every index is clamped
// into the arrays, so deeper ghost layers (partial tiles, corners) read
// valid memory; they never feed a face that is used.
template <typename R, int LAYOUT>
__device__ __forceinline__ void fetch_cell(const StepParams& P, int n, int m, R v[4])
{
    const int N = P.N, M = P.M;
    if (n >= 0 && n < N && m >= 0 && m < M) {
        read_cell<R, LAYOUT>(P, n, m, v);
        return;
    }
    int side, j, bn, bm, mn, mm;
    bool low;
    if (n < 0)       { side = 0; j = -1 - n; low = true;  bn = 0;     bm = m; mn = j;         mm = m; }
    else if (n >= N) { side = 1; j = n - N;  low = false; bn = N - 1; bm = m; mn = N - 1 - j; mm = m; }
    else if (m < 0)  { side = 2; j = -1 - m; low = true;  bn = n; bm = 0;     mn = n; mm = j; }
    else             { side = 3; j = m - M;  low = false; bn = n; bm = M - 1; mn = n; mm = M - 1 - j; }
    mn = min(max(mn, 0), N - 1);
    mm = min(max(mm, 0), M - 1);
    bm = min(max(bm, 0), M - 1);
    bn = min(max(bn, 0), N - 1);
    const int kind = P.bc_kind[side];
    const bool zside = side < 2;
    if (kind == 0) {            // REFLECT
        read_cell<R, LAYOUT>(P, mn, mm, v);
        if (zside) v[2] = -v[2]; else v[3] = -v[3];
    } else if (kind == 2) {     // FIXED
        v[0] = (R)P.bc_val[side][0]; v[1] = (R)P.bc_val[side][1];
        v[2] = (R)P.bc_val[side][2]; v[3] = (R)P.bc_val[side][3];
    } else {                    // OUTFLOW, SUCTION, NONREFLECT
        read_cell<R, LAYOUT>(P, bn, bm, v);
        if (kind == 3) {
            ghost_suction(zside, low, (R)(zside ? P.bc_val[side][2] : P.bc_val[side][3]), v);
        } else if (kind == 4) {
            ghost_nonreflect(gas_of<R>(P), zside, low, v);
        }
    }
}

__device__ __forceinline__ bool cell_fixed(const StepParams& P, double x, double y)
{
    double xz = x - P.fixed_zc;
    return (xz * xz) / P.fixed_az2 + (y * y) / P.fixed_ar2 < 1.0;
}

// ------------------------------------------------------------------ reductions
template <typename T>
__device__ __forceinline__ T warp_max(T v)
{
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// the four flux components of one face in shared memory: one 16-byte
// access in FP32, two in FP64
__device__ __forceinline__ void put4(float* d, float a, float b, float c, float e)
{
    *reinterpret_cast<float4*>(d) = make_float4(a, b, c, e);
}
__device__ __forceinline__ void put4(double* d, double a, double b, double c, double e)
{
    reinterpret_cast<double2*>(d)[0] = make_double2(a, b);
    reinterpret_cast<double2*>(d)[1] = make_double2(c, e);
}
__device__ __forceinline__ void get4(const float* s, float& a, float& b, float& c, float& e)
{
    const float4 t = *reinterpret_cast<const float4*>(s);
    a = t.x; b = t.y; c = t.z; e = t.w;
}
__device__ __forceinline__ void get4(const double* s, double& a, double& b, double& c, double& e)
{
    const double2 t0 = reinterpret_cast<const double2*>(s)[0], t1 = reinterpret_cast<const double2*>(s)[1];
    a = t0.x; b = t0.y; c = t1.x; e = t1.y;
}

// ------------------------------------------------------------------ shared memory of a tile
// The staged tile: NB buffers of the four planes, each TR+4 rows of TZ+8
// cells.  Cell (n, m) of the tile at (n0, m0) sits at row m - m0 + 2 and
// column n - n0 + 4 = i + QX, where i = n - n0 + 2 is the cell's index in
// the two-cell halo; the two extra columns on either side make the row
// start 16-byte aligned in global memory (n0 - 4 is a multiple of 4), so a
// TMA box can fill the buffer.
template <typename R, int TZ, int TR, int NB>
struct TileCore {
    static constexpr int HZ = TZ + 4, HR = TR + 4, HZP = TZ + 8, QX = 2;
    static constexpr int kNFZ = TR * (TZ + 1);                 // z faces of the tile
    static constexpr int kQueueCap = kNFZ + (TR + 1) * TZ;    // all faces of the tile
    alignas(128) R qb[NB][4][HR][HZP];   // staged state with a two-cell halo
    // face fluxes, the four components of a face contiguous (one 16-byte
    // access per face in FP32): z faces mass, mom_z, mom_r, energy; r faces
    // in the same order
    alignas(16) R Fz[TR][TZ + 1][4];
    alignas(16) R Fr[TR + 1][TZ][4];
    unsigned char fx[HR][HZ];    // 1 = cell held fixed (fixed_region only)
    unsigned qn;                 // queued faces: above the gate (low 16 bits), others (high 16 bits)
    double ydrow[TR];            // r of the tile's cell rows, y_min + m dy, in FP64
    float yfrow[TR];             // and in FP32
    double tydrow[TR];           // T_do / r of the rows (axisymmetric grid; FP64 kernels)
    float tyfrow[TR];            // and in FP32 (FP32 kernels with the step's constants set before the tile)
};

// the exact solver's queue: faces as 16-bit codes (face index | active <<
// 12 | pattern << 14); faces above the learned-start gate fill it from the
// front, the others from the back, so the two kinds sit in separate warps
template <typename R, int TZ, int TR>
struct QueueSmem {
    static constexpr int kCap = TR * (TZ + 1) + (TR + 1) * TZ;
    static_assert(kCap <= 4096, "face index fits 12 bits");
    unsigned short qcode[kCap];
};
template <int K>
struct Empty {};

// the start-value network in the queue phase: its vector block, W1 and W2
// as per-lane f16 mma fragments, and per warp the standardised features
// and outputs of 16 faces
struct NetSmem {
    float v[kVLen];
    unsigned B1[tc::kL1];
    unsigned B2[tc::kL2];
    float X[kThreads / 32][16][8];
    float Y[kThreads / 32][16];
};
static_assert(offsetof(NetSmem, B1) == sizeof(float) * kVLen &&
                  offsetof(NetSmem, B2) == sizeof(float) * (kVLen + tc::kL1),
              "v, B1 and B2 are the packed network's layout");

// the output tile of the TMA kernel (the updated cells, four dense planes)
// and the network's space: the network is used in the queue phase, before
// the update writes the output tile, and the previous tile's store has
// read the output tile before the next tile's faces start, so the two share
// memory
template <typename R, int TZ, int TR, bool OUT, bool NET>
struct OutNet;
template <typename R, int TZ, int TR>
struct OutNet<R, TZ, TR, false, false> {};
template <typename R, int TZ, int TR>
struct OutNet<R, TZ, TR, true, false> {
    alignas(128) R out[4][TR][TZ];
};
template <typename R, int TZ, int TR>
struct OutNet<R, TZ, TR, false, true> {
    NetSmem net;
};
template <typename R, int TZ, int TR>
struct OutNet<R, TZ, TR, true, true> {
    union {
        alignas(128) R out[4][TR][TZ];
        NetSmem net;
    };
};

template <typename R, int FLUX, int TZ, int TR, int NB = 1>
struct TileSmem : TileCore<R, TZ, TR, NB>,
                  std::conditional_t<FLUX == 2, QueueSmem<R, TZ, TR>, Empty<0>>,
                  OutNet<R, TZ, TR, (NB > 1), FLUX == 2> {
};

// dynamic shared memory of a kernel: the tile plus 128 bytes to align it
template <typename R, int FLUX, int TZ, int TR, int NB = 1>
constexpr size_t tile_smem_bytes() { return sizeof(TileSmem<R, FLUX, TZ, TR, NB>) + 128; }

template <typename S>
__device__ __forceinline__ S& tile_smem()
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const size_t a = reinterpret_cast<size_t>(smem_raw);
    return *reinterpret_cast<S*>(smem_raw + ((128 - (a & 127)) & 127));
}

// ------------------------------------------------------------------ cell update
// Conservative update of one cell in arithmetic C from its state `in`
// (rho, p, vz, vr) and its four face fluxes f[k][face] (k = mass, mom_z,
// mom_r, energy; face = right, left, bottom, top, all oriented along +z/+r).
// tdv = T_do/(dx dy), ty = T_do/r.  Planar: Kernel_TVD, kernel.cu:3027-3073;
// axisymmetric with the cylindrical source: add_MK, kernel.cu:2480-2509.
template <typename C, typename R>
__device__ __forceinline__ void update_cell(const StepParams& P, C ga, C g1, C inv_g1, const R in[4],
                                            const R f[4][4], C T_do, C tdv, C ty, C dx, C dy, C Q2, C Sz, C Sr,
                                            int& nrho, int& np, unsigned& status, R out[4], C* E2o = nullptr,
                                            C* KE2o = nullptr)
{
    const C r1 = (C)in[0], p1 = (C)in[1], vz1 = (C)in[2], vr1 = (C)in[3];
    C ps[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const C f12 = (C)f[k][0], f14 = -(C)f[k][1], f13 = -(C)f[k][2], f15 = (C)f[k][3];
        if (P.geom == 1) ps[k] = (f12 + f14) * dy + (f13 + f15) * dx;
        else ps[k] = f12 * dy + f13 * dx + f14 * dy + f15 * dx;
    }
    const C Q3 = Q2 * vr1;
    const C ke1 = r1 * (vz1 * vz1 + vr1 * vr1) * C(0.5);
    C rho2, mz, mr, E2;
    if (P.geom == 1) {
        rho2 = r1 - tdv * ps[0] - ty * r1 * vr1;
        if (rho2 <= C(0)) { nrho++; rho2 = r1; }
        mz = r1 * vz1 - tdv * ps[1] - ty * r1 * vr1 * vz1 + Sz;
        mr = r1 * vr1 - tdv * ps[2] - ty * r1 * vr1 * vr1 + T_do * Q2 + Sr;
        E2 = (p1 * inv_g1 + ke1) - tdv * ps[3] - ty * vr1 * (ga * p1 * inv_g1 + ke1) + T_do * Q3;
    } else {
        rho2 = r1 - tdv * ps[0];
        if (rho2 <= C(0)) { nrho++; rho2 = r1; }
        mz = r1 * vz1 - tdv * ps[1] + Sz;
        mr = r1 * vr1 - tdv * ps[2] + T_do * Q2 + Sr;
        E2 = (p1 * inv_g1 + ke1) - tdv * ps[3] + T_do * Q3;
    }
    const C irho = C(1) / rho2;
    const C vz2 = mz * irho, vr2 = mr * irho;
    const C KE2 = C(0.5) * rho2 * (vz2 * vz2 + vr2 * vr2);
    C p2 = (E2 - KE2) * g1;
    if (p2 <= C(0)) { np++; p2 = sizeof(C) == 4 ? (C)P.p_floorf : (C)P.p_floor; }
    // a non-finite flux or state reaches p2 through the energy or 1/rho
    // (a NaN sound speed can leave the wave speed finite: fmax drops NaN)
    if (!(p2 == p2)) status |= 0x10u;
    out[0] = (R)rho2; out[1] = (R)p2; out[2] = (R)vz2; out[3] = (R)vr2;
    if (E2o) { *E2o = E2; *KE2o = KE2; }
}

// The neutral-coupling source of cell (n, m): SoA planes of the state's
// precision (the solver's copy) or the reference's double3 array (raw
// entry points, AoS layout)
template <typename R, int LAYOUT, bool TO_SMEM, typename C>
__device__ __forceinline__ void neutral_at(const StepParams& P, int n, int m, C& az, C& ar)
{
    if constexpr (LAYOUT == kSoA || TO_SMEM) {
        const R* q = (const R*)P.nsrc + (long long)m * P.ld + n;
        az = (C)__ldg(q);
        ar = (C)__ldg(q + P.plane);
    } else {
        const double* q = (const double*)P.nsrc + 3 * ((long long)m * P.N + n);
        az = (C)__ldg(q);
        ar = (C)__ldg(q + 1);
    }
}

// The pressure of an updated FP32 cell recovered in FP64, for cells whose
// kinetic energy is almost all of the total (there p = (g-1)(E - rho v^2/2)
// cancels, and the FP32 E and rho v^2/2 leave too few bits).  The cell's
// increments (flux sums and sources, as update_cell forms them) are small
// against the state, so they are taken in FP32; the state, the updated
// conserved sums and the recovery run in FP64.  1/rho: the FP32 reciprocal
// refined by one Newton step in FP64 (relative error ~1e-14).
template <typename R>
__device__ __forceinline__ double pressure_fp64(const StepParams& P, const R in[4], const R f[4][4], float tdv,
                                                float ty, float T_do, float Q2, float dx, float dy, int& np)
{
    const float r1 = (float)in[0], p1 = (float)in[1], vz1 = (float)in[2], vr1 = (float)in[3];
    float ps[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float f12 = (float)f[k][0], f14 = -(float)f[k][1], f13 = -(float)f[k][2], f15 = (float)f[k][3];
        if (P.geom == 1) ps[k] = (f12 + f14) * dy + (f13 + f15) * dx;
        else ps[k] = f12 * dy + f13 * dx + f14 * dy + f15 * dx;
    }
    const float ke1 = r1 * (vz1 * vz1 + vr1 * vr1) * 0.5f;
    const float gaf = P.gf.ga, ig1f = P.gf.inv_g1;
    float dr = -tdv * ps[0], dmz = -tdv * ps[1], dmr = -tdv * ps[2] + T_do * Q2, dE = -tdv * ps[3] + T_do * Q2 * vr1;
    if (P.geom == 1) {
        dr -= ty * r1 * vr1;
        dmz -= ty * r1 * vr1 * vz1;
        dmr -= ty * r1 * vr1 * vr1;
        dE -= ty * vr1 * (gaf * p1 * ig1f + ke1);
    }
    const double R1 = r1, VZ = vz1, VR = vr1;
    const double E1 = (double)p1 * P.gd.inv_g1 + 0.5 * R1 * (VZ * VZ + VR * VR);
    double rho2 = R1 + (double)dr;
    if (rho2 <= 0.0) rho2 = R1;
    const double mz = R1 * VZ + (double)dmz, mr = R1 * VR + (double)dmr;
    const double E2 = E1 + (double)dE;
    double ir = (double)__frcp_rn((float)rho2);
    ir = fma(ir, fma(-rho2, ir, 1.0), ir);
    const double p2 = (E2 - 0.5 * (mz * mz + mr * mr) * ir) * P.gd.g1;
    if (p2 <= 0.0) { np++; return P.p_floor; }
    return p2;
}

// ------------------------------------------------------------------ exact solver helpers
// the face's own left/right states (before the solver's side swap)
template <typename R>
__device__ __forceinline__ void face_sides(const RPre<R>& q, R& rL, R& pL, R& uL, R& cL, R& rR, R& pR, R& uR, R& cR)
{
    rL = q.swap ? q.rII : q.rI; pL = q.swap ? q.pII : q.pI; cL = q.swap ? q.cII : q.cI;
    uL = q.swap ? -q.enII : q.enI;
    rR = q.swap ? q.rI : q.rII; pR = q.swap ? q.pI : q.pII; cR = q.swap ? q.cI : q.cII;
    uR = q.swap ? -q.enI : q.enII;
}

// wave strength of a face: max(|ln(p_R/p_L)|, |u_R - u_L| / min(c_L, c_R))
template <typename R>
__device__ __forceinline__ float wave_strength(const RPre<R>& q)
{
    const float lp = __logf((float)(q.pII / q.pI));
    const float du = fabsf((float)(q.enI - q.enII)) / (float)fmin(q.cI, q.cII);
    return fmaxf(lp, du);
}

// p* of a queued (pattern 2 or 3) face: the reference's iteration, or the
// safeguarded Newton.  Faces above the gate start from the learned value
// p0_mlp when the learned form is on (when it leaves the basin: from the
// acoustic value, counted as a fallback); all other faces start from the
// acoustic value.  Faces above the gate are counted in both forms, so the
// two start values can be compared on the same faces.
template <typename R>
__device__ __forceinline__ R solve_queued(const StepParams& P, const Gas<R>& g, const RPre<R>& q, bool strong,
                                          R p0_mlp, RiemannCount& rc, int& fallback)
{
    // the reference's own iteration (FP64 only: the FP32 form always runs
    // the safeguarded Newton, and its kernels leave this code out)
    if constexpr (sizeof(R) == 8) {
        if (!P.riemann_newton) return solve_p_reference(g, q, rc);
    }
    R p0;
    if (P.guess == 1 && strong) {
        p0 = p0_mlp;
        if (!in_basin(q, p0)) {
            fallback++;
            p0 = pvrs_guess(q);
        }
    } else {
        p0 = pvrs_guess(q);
    }
    const int k0 = rc.newton_iters;
    const R p = solve_p_newton(g, q, p0, g.tol, rc);
    if (strong) {
        rc.strong_calls++;
        rc.strong_iters += rc.newton_iters - k0;
    }
    return p;
}

// one training record of a solved face (recorder enabled)
template <typename R>
__device__ __forceinline__ void record_face(const StepParams& P, const Gas<R>& g, const RPre<R>& q, R p, int step,
                                            int face_id)
{
    const R rL = q.swap ? q.rII : q.rI, pL = q.swap ? q.pII : q.pI, cL = q.swap ? q.cII : q.cI;
    const R uL = q.swap ? -q.enII : q.enI;
    const R rR = q.swap ? q.rI : q.rII, pR = q.swap ? q.pI : q.pII, cR = q.swap ? q.cI : q.cII;
    const R uR = q.swap ? -q.enI : q.enII;
    if (P.rec_gate > 0.0 && !(wave_strength(q) > R(P.rec_gate))) return;
    const unsigned long long slot = atomicAdd(P.rec_n, 1ull);
    if ((long long)slot >= P.rec_cap) return;
    float* r = P.rec + slot * AST_RECORD_FLOATS;
    r[0] = (float)(rR / rL);
    r[1] = (float)(pR / pL);
    r[2] = (float)((uR - uL) / cL);
    r[3] = (float)(cR / cL);
    r[4] = (float)g.ga;
    r[5] = (float)log(pL);
    r[6] = (float)log(p / pL);
    r[7] = __int_as_float(step);
    r[8] = __int_as_float(face_id);
    r[9] = __int_as_float(q.pattern);
}

// ------------------------------------------------------------------ face passes
// bitwise equality of two staged values
__device__ __forceinline__ bool same_bits(float a, float b) { return __float_as_uint(a) == __float_as_uint(b); }
// a > 0 or a positive NaN, on the bit pattern
__device__ __forceinline__ bool positive_bits(float a) { return __float_as_int(a) > 0; }
__device__ __forceinline__ bool positive_bits(double a) { return __double_as_longlong(a) > 0; }
__device__ __forceinline__ bool same_bits(double a, double b)
{
    return __double_as_longlong(a) == __double_as_longlong(b);
}

// The reconstructed states on both sides of face (a, c) of orientation ZF
// (minmod on the staged cells when RECON and the face is in the
// high-order region `hi`; the cell values otherwise).  When the four
// stencil cells of every variable hold the same bits in all the warp's
// active lanes (undisturbed gas), the limited slope is +0 (x - x = +0, and
// minmod of zeros, or of the NaN of inf - inf, is +0), so the face values
// are the cell's value plus +0 and the upper cell's value: taken without
// the minmod arithmetic, the same bits.  (At step 1000 of the 4096x2048
// blast about nine faces in ten are such: the exact-solver step 0.189 ->
// 0.175 ms in FP32, 11.45 -> 10.44 ms in FP64; where the gas is disturbed
// everywhere the test costs about 5%.)  Returns whether the warp took
// that path (then the two sides of every lane's face are equal).
template <typename R, bool RECON, bool ZF, bool VOTE = true, typename S>
__device__ __forceinline__ bool face_states(const StepParams& P, const S& sm, int b, int a, int c, bool hi, R L[4],
                                            R U[4])
{
    constexpr int DJ = ZF ? 0 : 1, DI = ZF ? 1 : 0, QX = S::QX;
    // buffer indices of the lower (l) and upper (u) cell of the face
    const int jl = ZF ? a + 2 : a + 1, il = (ZF ? c + 1 : c + 2) + QX;
    const int ju = a + 2, iu = c + 2 + QX;
    const auto& q = sm.qb[b];
    R tl[4], tu[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        tl[k] = q[k][jl][il];
        tu[k] = q[k][ju][iu];
        L[k] = tl[k];
        U[k] = tu[k];
    }
    if (RECON && hi) {
        R tll[4], tuu[4];
        bool flat = true;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            tll[k] = q[k][jl - DJ][il - DI];
            tuu[k] = q[k][ju + DJ][iu + DI];
            flat = flat && same_bits(tll[k], tl[k]) && same_bits(tl[k], tu[k]) && same_bits(tu[k], tuu[k]);
        }
        if (VOTE && __all_sync(__activemask(), flat)) {
#pragma unroll
            for (int k = 0; k < 4; k++) L[k] = tl[k] + R(0);
            // (the positivity rule below leaves equal sides equal)
            if (L[0] <= R(0)) L[0] = tl[0];
            if (L[1] <= R(0) || !P.grad_p) L[1] = tl[1];
            return true;
        } else {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                R x0, x1;
                recon_pair(tll[k], tl[k], tu[k], x0, x1);
                L[k] = x1;                  // right/top value of the lower cell
                recon_pair(tl[k], tu[k], tuu[k], x0, x1);
                U[k] = x0;                  // left/bottom value of the upper cell
            }
        }
        // positivity of the reconstructed rho and p (kernel.cu:2706-2743)
        if (L[0] <= R(0)) L[0] = tl[0];
        if (U[0] <= R(0)) U[0] = tu[0];
        if (L[1] <= R(0) || !P.grad_p) L[1] = tl[1];
        if (U[1] <= R(0) || !P.grad_p) U[1] = tu[1];
    }
    return false;
}

// Whether face (a, c) of orientation ZF belongs to an updated cell
// (active: its wave speed counts for dt) and lies in the high-order region
// (hi).  ZF: z faces (between tile columns c-1 and c of row a), else r
// faces (between tile rows a-1 and a of column c).
template <int TZ, int TR, bool ZF, typename S>
__device__ __forceinline__ void face_meta(const StepParams& P, const S& sm, int n0, int m0, bool interior, int a,
                                          int c, bool& active, bool& hi)
{
    // smem indices of the lower (l) and upper (u) cell of the face
    const int jl = ZF ? a + 2 : a + 1, il = ZF ? c + 1 : c + 2;
    const int ju = a + 2, iu = c + 2;
    // both cells inside the grid (always so in an interior tile)
    bool lval = true, uval = true;
    if (!interior) {
        const int nl = n0 + il - 2, ml = m0 + jl - 2, nu = n0 + iu - 2, mu = m0 + ju - 2;
        lval = nl >= 0 && nl < P.N && ml >= 0 && ml < P.M;
        uval = nu >= 0 && nu < P.N && mu >= 0 && mu < P.M;
    }
    active = lval || uval;
    if (active && P.fixed_region) active = (lval && !sm.fx[jl][il]) || (uval && !sm.fx[ju][iu]);
    hi = true;
    if (P.region_select) {
        // the face's z position as the reference's lower cell sees it, as an
        // interval of that cell's column (integer compares: an FP64 position
        // test here ran on every face, region or not)
        const int nl = n0 + il - 2;
        hi = ZF ? (nl >= P.region_zlo && nl <= P.region_zhi) : (nl >= P.region_rlo && nl <= P.region_rhi);
    }
}

// The flux of face (a, c) from its reconstructed states L (lower cell) and U
// (upper cell): written, in (mass, mom_z, mom_r, energy) order, to sm.Fz /
// sm.Fr, and smax raised to its wave speed when the face is active.
// Exact-solver faces of patterns 2 and 3 go to the queue instead.
template <typename R, int FLUX, int TZ, int TR, bool ZF, typename S>
__device__ __forceinline__ void face_flux(const StepParams& P, S& sm, const Gas<R>& g, int a, int c, bool active,
                                          bool hi, const R L[4], const R U[4], RiemannCount& rc, R& smax,
                                          bool same_sides = false)
{
    constexpr int NFZ = TR * (TZ + 1);
    constexpr int W = ZF ? TZ + 1 : TZ;      // faces per row of the face array
    constexpr int NN = ZF ? 2 : 3;           // normal velocity component
    constexpr int TT = ZF ? 3 : 2;           // tangential velocity component
    R F[4];
    R Sp;
    // FP64, the HLL or HLLC flux, the faces of every active lane of the warp
    // with one state (one bit pattern, rho > 0, p > 0) on both sides
    // (undisturbed gas): that state's physical flux (flux_physical; the
    // solvers' formulas give it up to rounding) for two divisions, two square
    // roots and the star-state arithmetic.  A warp vote, so that warps with
    // other faces run as before; bit tests, not FP64 compares (this GPU's
    // FP64 pipe is slow).
    bool same = false;
    if constexpr (sizeof(R) == 8 && FLUX != 2) {
        const bool eq = (FLUX == 0 || FLUX == 1 || !hi) && same_bits(L[0], U[0]) && same_bits(L[1], U[1]) &&
                        same_bits(L[2], U[2]) && same_bits(L[3], U[3]) && positive_bits(L[0]) &&
                        positive_bits(L[1]);
        if (__all_sync(__activemask(), eq)) {
            Sp = flux_physical(g, L[0], L[1], L[NN], L[TT], F);
            same = true;
        }
    }
    if (same) {
    } else if constexpr (FLUX == 2) {
        if (!active) {
            // no updated cell uses this face (both cells outside the grid or
            // held fixed): not solved, so the solver's counters see the same
            // faces however the tile was staged
            F[0] = F[1] = F[2] = F[3] = R(0);
            Sp = R(0);
        } else if (hi && (same_sides || (L[0] == U[0] && L[1] == U[1] && L[2] == U[2] && L[3] == U[3]))) {
            // identical states: the exact solution is that state (the
            // reference reaches it through the two-rarefaction branch with
            // p* = p, u* = u_n, up to rounding), its flux the physical flux
            // and its largest wave speed |u_n| + c
            const R r = L[0], p = L[1], un = L[NN], ut = L[TT];
            const R cs = sqrt(g.ga * p / r);
            const R m = r * un;
            F[0] = m;
            F[1] = m * un + p;
            F[2] = m * ut;
            F[3] = un * (p * g.inv_g1 + R(0.5) * r * (un * un + ut * ut) + p);
            Sp = fmax(fabs(un) + cs, g.eps8);
            // stored here: fmax drops a NaN, so this wave speed needs no
            // test for one
            if (ZF) put4(sm.Fz[a][c], F[0], F[1], F[2], F[3]);
            else put4(sm.Fr[a][c], F[0], F[2], F[1], F[3]);
            if (active) smax = fmax(smax, Sp);
            return;
        } else if (hi) {
            const RPre<R> q = godunov_pre(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT]);
            if (q.pattern == 2 || q.pattern == 3) {
                // the iterative faces go to the queue (room for every face
                // of the tile); their flux is written by queue_pass
                const bool strong = P.riemann_newton && wave_strength(q) > P.mlp_gate;
                const unsigned old = atomicAdd(&sm.qn, strong ? 1u : 0x10000u);
                const int slot = strong ? (int)(old & 0xffffu) : S::kQueueCap - 1 - (int)(old >> 16);
                const int f = a * W + c;
                sm.qcode[slot] = (unsigned short)((ZF ? f : NFZ + f) | (active ? 1 << 12 : 0) | (q.pattern << 14));
                return;
            }
            Sp = godunov_sample<R, kSampleClosed>(g, q, R(0), F, rc);
        } else {
            Sp = flux_hll(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT], F);
        }
    } else if constexpr (FLUX == 1) {
        if (hi) Sp = flux_hllc(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT], F);
        else Sp = flux_hll(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT], F);
    } else if constexpr (FLUX == 3) {
        if (hi) Sp = flux_hllc_a(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT], F);
        else Sp = flux_hll(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT], F);
    } else if constexpr (FLUX == 4) {
        // HLLCQ_Korolkov_2D's gas part (the FP64 solver only)
        R FQ;
        if (hi) Sp = flux_hllcq(g, L[0], L[1], L[NN], L[TT], R(0), U[0], U[1], U[NN], U[TT], R(0), F, FQ);
        else Sp = flux_hll(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT], F);
    } else {
        Sp = flux_hll(g, L[0], L[1], L[NN], L[TT], U[0], U[1], U[NN], U[TT], F);
    }
    if (!(Sp == Sp)) { rc.status |= 0x10u; Sp = R(0); }
    if (ZF) {
        put4(sm.Fz[a][c], F[0], F[1], F[2], F[3]);
    } else {
        // r face: the normal momentum is mom_r, the tangential one mom_z
        put4(sm.Fr[a][c], F[0], F[2], F[1], F[3]);
    }
    if (active) smax = fmax(smax, Sp);
}

// Two adjacent faces of orientation ZF in one thread: (a, c) and the next
// one along the normal ((a, c + 1) for z faces, (a + 1, c) for r faces), or
// (a, c) alone when !two.  The five staged cells along the normal (the
// first face's lower cell's lower neighbour .. the second face's upper
// cell's upper neighbour) give the slopes of the three middle cells, each
// once, so the cell between the two faces is reconstructed once for both
// (minmod, linear2 and the positivity rule as face_states applies them, the
// same values).  Z faces take c even and load the cells as aligned pairs.
template <typename R, int FLUX, bool RECON, int TZ, int TR, bool ZF, bool FF = false, typename S>
__device__ __forceinline__ void face_two(const StepParams& P, S& sm, int b, const Gas<R>& g, int n0, int m0,
                                         bool interior, RiemannCount& rc, R& smax, int a, int c, bool two)
{
    constexpr int QX = S::QX, HR = S::HR;
    using R2 = std::conditional_t<sizeof(R) == 4, float2, double2>;
    const int a1 = ZF ? a : a + 1, c1 = ZF ? c + 1 : c;
    bool act0, hi0, act1 = false, hi1 = true;
    face_meta<TZ, TR, ZF>(P, sm, n0, m0, interior, a, c, act0, hi0);
    if (two) face_meta<TZ, TR, ZF>(P, sm, n0, m0, interior, a1, c1, act1, hi1);
    R L0[4], U0[4], L1[4], U1[4];
    const auto& q = sm.qb[b];
    // the five staged cells of variable k along the normal
    auto load5 = [&](int k, R v[5]) {
        if constexpr (ZF) {
            // row a, columns c-2 .. c+2 (smem columns c+QX .. c+QX+4, c+QX even)
            const R2 p0 = *reinterpret_cast<const R2*>(&q[k][a + 2][c + QX]);
            const R2 p1 = *reinterpret_cast<const R2*>(&q[k][a + 2][c + QX + 2]);
            const R2 p2 = *reinterpret_cast<const R2*>(&q[k][a + 2][c + QX + 4]);
            v[0] = p0.x; v[1] = p0.y; v[2] = p1.x; v[3] = p1.y; v[4] = p2.x;
        } else {
            // column c, rows a-2 .. a+2 (smem rows a .. a+4; the last
            // clamped into the buffer for a single face at the tile's top)
            v[0] = q[k][a][c + 2 + QX];
            v[1] = q[k][a + 1][c + 2 + QX];
            v[2] = q[k][a + 2][c + 2 + QX];
            v[3] = q[k][a + 3][c + 2 + QX];
            v[4] = q[k][min(a + 4, HR - 1)][c + 2 + QX];
        }
    };
    auto store = [&](int fa, int fc, bool act, R f0, R f1, R f2, R f3, R sp) {
        if (!(sp == sp)) { rc.status |= 0x10u; sp = R(0); }
        if (ZF) put4(sm.Fz[fa][fc], f0, f1, f2, f3);
        else put4(sm.Fr[fa][fc], f0, f2, f1, f3);
        if (act) smax = fmax(smax, sp);
    };
    // FF (kernels with the skip_uniform code, when it is set): HLL in FP32,
    // a face pair in the high-order region.  When the five staged cells of
    // every variable hold one bit pattern (rho, p > 0, velocities not -0) in
    // every active lane of the warp (undisturbed gas), every limited slope is
    // +0 and all four face values are the middle cell's value plus +0, so
    // both faces take that state's physical flux (as below, where the four
    // sides are found equal after the reconstruction: the same bits), with no
    // reconstruction.  The density is voted on first, the other variables
    // only when it is flat in the whole warp.  Measured at 4096x2048: the
    // blast at step 1000 0.1414 -> 0.1229 ms per step, but the wind problem
    // with HLL (its seeded noise disturbs every face) 0.0555 -> 0.0599 ms, so
    // it goes with the opt-in skip_uniform and not into the default kernel.
    constexpr bool kFlatFirst = FF && FLUX == 0 && sizeof(R) == 4 && RECON;
    R rho5[5];
    const bool ff = kFlatFirst && P.skip_uniform;
    if (kFlatFirst && ff) {
        constexpr int NN = ZF ? 2 : 3, TT = ZF ? 3 : 2;
        load5(0, rho5);
        bool flat = two && hi0 && hi1 && same_bits(rho5[0], rho5[1]) && same_bits(rho5[1], rho5[2]) &&
                    same_bits(rho5[2], rho5[3]) && same_bits(rho5[3], rho5[4]) && positive_bits(rho5[2]);
        if (__all_sync(__activemask(), flat)) {
            R st[4];
            st[0] = rho5[2];
#pragma unroll
            for (int k = 1; k < 4; k++) {
                R v[5];
                load5(k, v);
                flat = flat && same_bits(v[0], v[1]) && same_bits(v[1], v[2]) && same_bits(v[2], v[3]) &&
                       same_bits(v[3], v[4]);
                st[k] = v[2];
            }
            flat = flat && positive_bits(st[1]) && __float_as_uint(st[2]) != 0x80000000u &&
                   __float_as_uint(st[3]) != 0x80000000u;
            if (__all_sync(__activemask(), flat)) {
                R f[4];
                const R sp = flux_physical(g, st[0], st[1], st[NN], st[TT], f);
                store(a, c, act0, f[0], f[1], f[2], f[3], sp);
                store(a1, c1, act1, f[0], f[1], f[2], f[3], sp);
                return;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < 4; k++) {
        R v[5];
        load5(k, v);
        L0[k] = v[1]; U0[k] = v[2]; L1[k] = v[2]; U1[k] = v[3];
        if (RECON) {
            R x0, x1, y0, y1, z0, z1;
            // FP64: five cells of one bit pattern in every active lane of
            // the warp (undisturbed gas): every limited slope is +0, so the
            // face values are the cells' values plus or minus +0
            // (face_states).  (In FP32 the test costs what it saves: HLL
            // 0.150 ms per step either way at step 1000 of the blast; FP64
            // HLL 5.87 -> 5.20 ms.)
            bool flat = false;
            if constexpr (sizeof(R) == 8)
                flat = same_bits(v[0], v[1]) && same_bits(v[1], v[2]) && same_bits(v[2], v[3]) &&
                       same_bits(v[3], v[4]);
            if (sizeof(R) == 8 && __all_sync(__activemask(), flat)) {
                x1 = v[1] + R(0);
                y0 = v[2];
                y1 = v[2] + R(0);
                z0 = v[3];
            } else {
                recon_pair(v[0], v[1], v[2], x0, x1);   // lower cell of the first face
                recon_pair(v[1], v[2], v[3], y0, y1);   // the cell between the faces
                recon_pair(v[2], v[3], v[4], z0, z1);   // upper cell of the second face
            }
            if (hi0) { L0[k] = x1; U0[k] = y0; }
            if (hi1) { L1[k] = y1; U1[k] = z0; }
            // positivity of the reconstructed rho and p (kernel.cu:2706-2743)
            if (k == 0) {
                if (L0[0] <= R(0)) L0[0] = v[1];
                if (U0[0] <= R(0)) U0[0] = v[2];
                if (L1[0] <= R(0)) L1[0] = v[2];
                if (U1[0] <= R(0)) U1[0] = v[3];
            } else if (k == 1) {
                if (L0[1] <= R(0) || !P.grad_p) L0[1] = v[1];
                if (U0[1] <= R(0) || !P.grad_p) U0[1] = v[2];
                if (L1[1] <= R(0) || !P.grad_p) L1[1] = v[2];
                if (U1[1] <= R(0) || !P.grad_p) U1[1] = v[3];
            }
        }
    }
    if constexpr (FLUX == 0 && sizeof(R) == 4) {
        // HLL in FP32: both faces in packed arithmetic; or, when both faces
        // of every active lane of the warp hold one state on all four sides
        // (one bit pattern, rho > 0, p > 0: undisturbed gas), that state's
        // physical flux once for both (flux_physical: what the HLL formula
        // gives up to rounding, its wave speed formed as the formula forms it)
        constexpr int NN = ZF ? 2 : 3, TT = ZF ? 3 : 2;
        float2 F[4], Sp;
        bool one = two && positive_bits(L0[0]) && positive_bits(L0[1]);
#pragma unroll
        for (int k = 0; k < 4; k++)
            one = one && same_bits(L0[k], U0[k]) && same_bits(L0[k], L1[k]) && same_bits(L0[k], U1[k]);
        if (__all_sync(__activemask(), one)) {
            float f[4];
            const float s = flux_physical(g, L0[0], L0[1], L0[NN], L0[TT], f);
#pragma unroll
            for (int k = 0; k < 4; k++) F[k] = pk(f[k], f[k]);
            Sp = pk(s, s);
        } else {
            flux_hll_x2(g, pk(L0[0], L1[0]), pk(L0[1], L1[1]), pk(L0[NN], L1[NN]), pk(L0[TT], L1[TT]),
                        pk(U0[0], U1[0]), pk(U0[1], U1[1]), pk(U0[NN], U1[NN]), pk(U0[TT], U1[TT]), F, Sp);
        }
        store(a, c, act0, F[0].x, F[1].x, F[2].x, F[3].x, Sp.x);
        if (two) store(a1, c1, act1, F[0].y, F[1].y, F[2].y, F[3].y, Sp.y);
    } else {
        // one flux call site for both faces (a smaller kernel)
#pragma unroll 1
        for (int s = 0; s < (two ? 2 : 1); s++) {
            face_flux<R, FLUX, TZ, TR, ZF>(P, sm, g, s ? a1 : a, s ? c1 : c, s ? act1 : act0, s ? hi1 : hi0, L0, U0,
                                           rc, smax);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                L0[k] = L1[k];
                U0[k] = U1[k];
            }
        }
    }
}

// Face (a, c) of orientation ZF alone: its states by face_states (the
// exact solver's face pass; its kernel is large enough that the two-face
// form's extra code costs more in instruction fetch than it saves).
template <typename R, int FLUX, bool RECON, int TZ, int TR, bool ZF, typename S>
__device__ __forceinline__ void face_one(const StepParams& P, S& sm, int b, const Gas<R>& g, int n0, int m0,
                                         bool interior, RiemannCount& rc, R& smax, int a, int c)
{
    bool active, hi;
    face_meta<TZ, TR, ZF>(P, sm, n0, m0, interior, a, c, active, hi);
    R L[4], U[4];
    const bool same = face_states<R, RECON, ZF>(P, sm, b, a, c, hi, L, U);
    face_flux<R, FLUX, TZ, TR, ZF>(P, sm, g, a, c, active, hi, L, U, rc, smax, same);
}

// every face of the tile once, in one loop over the CTA's threads.
// HLL / HLLC / HLLC_A: two adjacent faces per thread, first the z face
// pairs (c, c+1 for even c < TZ) of every row, then the r face pairs (rows
// a, a+1 for even a < TR) of every column, then the single faces left: the
// r faces of row TR and the z faces c = TZ (those last go to the first
// warps; the last warp holds the copy thread of the persistent kernel).
// Exact Godunov: one face per thread, the z faces c < TZ of each row (a warp
// per row when TZ = 32, so the warp's staged-cell loads hit distinct
// banks), then the last z face (c = TZ) of every row, then the r faces; each
// group padded to whole warps so that no warp mixes groups.
template <typename R, int FLUX, bool RECON, int TZ, int TR, bool FF = false, typename S>
__device__ __forceinline__ void face_pass(const StepParams& P, S& sm, int b, const Gas<R>& g, int n0, int m0,
                                          int step, RiemannCount& rc, int& fallback, R& smz, R& smr)
{
    // every cell the tile's faces touch lies inside the grid
    const bool interior = n0 >= 1 && n0 + TZ < P.N && m0 >= 1 && m0 + TR < P.M;
    if constexpr (FLUX != 2) {
        static_assert(TZ % 2 == 0 && TR % 2 == 0, "faces in pairs");
        constexpr int NZP = TR * (TZ / 2);          // z face pairs
        constexpr int NP = NZP + (TR / 2) * TZ;     // + r face pairs
        constexpr int TZP = (TZ + 31) / 32 * 32;    // r faces of row TR, padded to whole warps
        static_assert(NZP % 32 == 0 && NP % 32 == 0, "no warp mixes groups");
        for (int t = threadIdx.x; t < NP + TZP + TR; t += kThreads) {
            if (t < NZP) {
                const int a = t / (TZ / 2);
                face_two<R, FLUX, RECON, TZ, TR, true, FF>(P, sm, b, g, n0, m0, interior, rc, smz, a,
                                                       2 * (t - a * (TZ / 2)), true);
            } else if (t < NP) {
                const int u = t - NZP, a = u / TZ;
                face_two<R, FLUX, RECON, TZ, TR, false, FF>(P, sm, b, g, n0, m0, interior, rc, smr, 2 * a, u - a * TZ,
                                                        true);
            } else if (t < NP + TZ) {
                face_two<R, FLUX, RECON, TZ, TR, false, FF>(P, sm, b, g, n0, m0, interior, rc, smr, TR, t - NP, false);
            } else if (t >= NP + TZP) {
                face_two<R, FLUX, RECON, TZ, TR, true, FF>(P, sm, b, g, n0, m0, interior, rc, smz, t - NP - TZP, TZ,
                                                       false);
            }
        }
    } else {
        constexpr int NZM = TR * TZ;                               // z faces c < TZ
        constexpr int NZMP = (NZM + 31) / 32 * 32;
        constexpr int NZL = NZMP + TR, NZLP = NZMP + (TR + 31) / 32 * 32;   // + the last z face of each row
        constexpr int NFR = (TR + 1) * TZ;
        for (int t = threadIdx.x; t < NZLP + NFR; t += kThreads) {
            if (t < NZLP) {
                // one call site for both z groups (a smaller kernel)
                int a, c;
                if (t < NZM) {
                    a = t / TZ;
                    c = t - a * TZ;
                } else if (t >= NZMP && t < NZL) {
                    a = t - NZMP;
                    c = TZ;
                } else {
                    continue;
                }
                face_one<R, FLUX, RECON, TZ, TR, true>(P, sm, b, g, n0, m0, interior, rc, smz, a, c);
            } else {
                const int a = (t - NZLP) / TZ;
                face_one<R, FLUX, RECON, TZ, TR, false>(P, sm, b, g, n0, m0, interior, rc, smr, a,
                                                        t - NZLP - a * TZ);
            }
        }
    }
}

// the exact-solver states of queued face fc (z faces first, then r faces):
// its reconstructed sides, swapped as godunov_pre swaps them, with the
// pattern found in face_pass; lower/upper states in the face frame too
template <typename R, bool RECON, int TZ, int TR, typename S>
__device__ __forceinline__ RPre<R> queued_face(const StepParams& P, const S& sm, int b, const Gas<R>& g, int fc,
                                               int pattern, int& a, int& c, bool& zf)
{
    constexpr int NFZ = S::kNFZ;
    R L[4], U[4];
    zf = fc < NFZ;
    if (zf) {
        a = fc / (TZ + 1);
        c = fc - a * (TZ + 1);
        face_states<R, RECON, true, false>(P, sm, b, a, c, true, L, U);
    } else {
        a = (fc - NFZ) / TZ;
        c = (fc - NFZ) - a * TZ;
        face_states<R, RECON, false, false>(P, sm, b, a, c, true, L, U);
    }
    // normal and tangential velocity: (v_z, v_r) on z faces, (v_r, v_z) on r faces
    const R unL = zf ? L[2] : L[3], utL = zf ? L[3] : L[2];
    const R unU = zf ? U[2] : U[3], utU = zf ? U[3] : U[2];
    RPre<R> q = godunov_sides(g, L[0], L[1], unL, utL, U[0], U[1], unU, utU);
    q.pattern = pattern;
    return q;
}

// the queued exact-solver faces, solved by all threads of the CTA
template <typename R, bool RECON, int TZ, int TR, typename S>
__device__ __forceinline__ void queue_pass(const StepParams& P, S& sm, int b, const Gas<R>& g, int n0, int m0,
                                           int step, RiemannCount& rc, int& fallback, R& smz, R& smr)
{
    constexpr int CAP = S::kQueueCap;
    const int ns = (int)(sm.qn & 0xffffu), nw = (int)(sm.qn >> 16);
    if (P.riemann_newton && P.guess == 1 && P.mlp != nullptr && ns > 0) {
        // phase 1: learned start values of the faces above the gate (queue
        // slots 0..ns-1), 16 per warp tile on the tensor cores.  Only tiles
        // with such faces stage the network: its packed form (written after
        // the parameters on upload) by 16-byte asynchronous copies, no
        // registers in between.  A face's start value waits in its own flux
        // slot (written with the flux in phase 2).
        {
            const char* src = reinterpret_cast<const char*>(P.mlp + kMlpPackOff);
            char* dst = reinterpret_cast<char*>(&sm.net.v[0]);
            for (int i = threadIdx.x; i < kMlpPackWords / 4; i += kThreads)
                tma::async_copy16(dst + 16 * i, src + 16 * i);
            tma::async_commit();
            tma::async_wait_all();
        }
        __syncthreads();
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        for (int t0 = 16 * w; t0 < ns; t0 += 16 * (kThreads / 32)) {
            const int i = t0 + (lane & 15);
            R pL = R(1);
            R* p0_slot = nullptr;
            if (lane < 16) {
                float x[kMlpIn] = {0, 0, 0, 0, 0, 0};
                if (i < ns) {
                    const int code = sm.qcode[i];
                    int a, c;
                    bool zf;
                    const RPre<R> q =
                        queued_face<R, RECON, TZ, TR>(P, sm, b, g, code & 0xfff, (code >> 14) & 3, a, c, zf);
                    R rL, uL, cL, rR, pR, uR, cR;
                    face_sides(q, rL, pL, uL, cL, rR, pR, uR, cR);
                    mlp_features((float)g.ga, (float)rL, (float)pL, (float)uL, (float)cL, (float)rR, (float)pR,
                                 (float)uR, (float)cR, x);
                    p0_slot = zf ? &sm.Fz[a][c][0] : &sm.Fr[a][c][0];
                }
                // standardised, and clamped to a range f16 holds exactly enough
#pragma unroll
                for (int k = 0; k < kMlpIn; k++)
                    sm.net.X[w][lane][k] =
                        fminf(fmaxf((mlp_map(k, x[k]) - sm.net.v[kVShift + k]) * sm.net.v[kVScale + k], -30.0f),
                              30.0f);
                sm.net.X[w][lane][6] = 0.0f;
                sm.net.X[w][lane][7] = 0.0f;
            }
            __syncwarp();
            tc::forward16(sm.net.v, sm.net.B1, sm.net.B2, sm.net.X[w], sm.net.Y[w]);
            __syncwarp();
            if (p0_slot) *p0_slot = pL * (R)__expf(sm.net.Y[w][lane]);
            __syncwarp();
        }
        __syncthreads();
    }
    // phase 2: p* (iteration), sampling and the flux of each queued face;
    // threads 0..ns-1 take the faces above the gate
    for (int t = threadIdx.x; t < ns + nw; t += kThreads) {
        const bool strong = t < ns;
        const int i = strong ? t : CAP - 1 - (t - ns);
        const int code = sm.qcode[i];
        const bool active = (code >> 12) & 1;
        int a, c;
        bool zf;
        const RPre<R> q = queued_face<R, RECON, TZ, TR>(P, sm, b, g, code & 0xfff, (code >> 14) & 3, a, c, zf);
        // a gated face's learned start value, left in its flux slot by phase 1
        const R p0 = (strong && P.guess == 1 && P.mlp) ? (zf ? sm.Fz[a][c][0] : sm.Fr[a][c][0]) : R(0);
        const R p = solve_queued(P, g, q, strong, p0, rc, fallback);
        R F[4];
        R Sp = godunov_sample<R, kSampleIterative>(g, q, p, F, rc);
        if (!(Sp == Sp)) { rc.status |= 0x10u; Sp = R(0); }
        if (zf) {
            put4(sm.Fz[a][c], F[0], F[1], F[2], F[3]);
            if (active) smz = fmax(smz, Sp);
        } else {
            put4(sm.Fr[a][c], F[0], F[2], F[1], F[3]);
            if (active) smr = fmax(smr, Sp);
        }
        // the recorder runs on the FP64 solver only (its records are training
        // targets; the FP32 kernels are smaller without it)
        if constexpr (sizeof(R) == 8) {
            if (P.rec && step % P.rec_every == 0)
                record_face(P, g, q, p, step, 2 * ((m0 + a) * P.N + (n0 + c)) + (zf ? 0 : 1));
        }
    }
}

// ------------------------------------------------------------------ one tile of one step
// per-thread running values over the tiles a CTA processes in one step
template <typename R>
struct TileAcc {
    RiemannCount rc;
    int fallback, nrho, np;
    R smz, smr;
    __device__ __forceinline__ void clear()
    {
        rc.clear();
        fallback = nrho = np = 0;
        smz = smr = R(0);
    }
};

// constants of the step every tile shares (set by thread 0, read after a barrier)
struct StepConsts {
    double T_do;           // the step's dt
    double tdv;            // T_do / (dx dy)
    float tdv_f, T_f;
    int step;
};

__device__ __forceinline__ void step_consts_of(const StepParams& P, double T_do, int step, StepConsts& K)
{
    K.T_do = T_do;
    K.step = step;
    K.tdv = K.T_do / (P.dx * P.dy);
    K.tdv_f = (float)K.tdv;
    K.T_f = (float)K.T_do;
}

__device__ __forceinline__ void step_consts(const StepParams& P, StepConsts& K)
{
    step_consts_of(P, (P.clock != nullptr) ? *(volatile double*)&P.clock->T_do : *P.T_do_ptr,
                   (P.clock != nullptr) ? (int)P.clock->step : 0, K);
}

// the fixed region's exact test (FP64 divisions, as the reference evaluates
// it) only in tiles whose cells, halo included, meet the region's cell
// bounding box
template <int TZ, int TR>
__device__ __forceinline__ bool tile_near_fixed(const StepParams& P, int n0, int m0)
{
    return P.fixed_region && n0 - 2 <= P.fixed_nhi && n0 + TZ + 1 >= P.fixed_nlo && m0 - 2 <= P.fixed_mhi;
}

// stage tile + halo from global memory into buffer b, ghost rules applied;
// the corners are never read by the cross stencil
template <typename R, int LAYOUT, int TZ, int TR, typename S>
__device__ __forceinline__ void stage_tile(const StepParams& P, S& sm, int b, int n0, int m0)
{
    constexpr int HZ = S::HZ, HR = S::HR, QX = S::QX;
    const bool near_fixed = tile_near_fixed<TZ, TR>(P, n0, m0);
    for (int idx = threadIdx.x; idx < HR * HZ; idx += kThreads) {
        const int j = idx / HZ, i = idx - j * HZ;
        const bool rin = (j >= 2 && j < TR + 2), cin = (i >= 2 && i < TZ + 2);
        if (!rin && !cin) continue;
        const int n = n0 - 2 + i, m = m0 - 2 + j;
        R v[4];
        fetch_cell<R, LAYOUT>(P, n, m, v);
        sm.qb[b][0][j][i + QX] = v[0]; sm.qb[b][1][j][i + QX] = v[1];
        sm.qb[b][2][j][i + QX] = v[2]; sm.qb[b][3][j][i + QX] = v[3];
        if (P.fixed_region) {
            const bool inside = (n >= 0 && n < P.N && m >= 0 && m < P.M);
            sm.fx[j][i] = (inside && near_fixed) ? (unsigned char)cell_fixed(P, P.x_min + n * P.dx, P.y_min + m * P.dy)
                                                 : 0;
        }
    }
}

// After a bulk copy of the tile box into buffer b (zeros outside the
// grid): the cross-stencil cells outside the grid get their ghost values
// from the staged cells, as fetch_cell gives them from global memory, for
// the two ghost layers next to the boundary; deeper ghost cells (those of a
// partial tile beyond its last row or column, which feed only faces that
// no updated cell uses) become copies of the boundary cell.  Also sets the
// fixed-region flags.
template <typename R, int TZ, int TR, typename S>
__device__ __forceinline__ void patch_tile_body(const StepParams& P, S& sm, int b, int n0, int m0)
{
    constexpr int HZ = S::HZ, HR = S::HR, QX = S::QX;
    const int N = P.N, M = P.M;
    const bool edge = n0 - 2 < 0 || n0 + TZ + 2 > N || m0 - 2 < 0 || m0 + TR + 2 > M;
    const bool near_fixed = tile_near_fixed<TZ, TR>(P, n0, m0);
    if (!edge && !P.fixed_region) return;
    auto& q = sm.qb[b];
    for (int idx = threadIdx.x; idx < HR * HZ; idx += kThreads) {
        const int j = idx / HZ, i = idx - j * HZ;
        const bool rin = (j >= 2 && j < TR + 2), cin = (i >= 2 && i < TZ + 2);
        if (!rin && !cin) continue;
        const int n = n0 - 2 + i, m = m0 - 2 + j;
        const bool inside = (n >= 0 && n < N && m >= 0 && m < M);
        if (P.fixed_region)
            sm.fx[j][i] = (inside && near_fixed) ? (unsigned char)cell_fixed(P, P.x_min + n * P.dx, P.y_min + m * P.dy)
                                                 : 0;
        if (inside) continue;
        int side, g, bn, bm, mn, mm;
        bool low;
        if (n < 0)       { side = 0; g = -1 - n; low = true;  bn = 0;     bm = m; mn = g;         mm = m; }
        else if (n >= N) { side = 1; g = n - N;  low = false; bn = N - 1; bm = m; mn = N - 1 - g; mm = m; }
        else if (m < 0)  { side = 2; g = -1 - m; low = true;  bn = n; bm = 0;     mn = n; mm = g; }
        else             { side = 3; g = m - M;  low = false; bn = n; bm = M - 1; mn = n; mm = M - 1 - g; }
        mn = min(max(mn, 0), N - 1);
        mm = min(max(mm, 0), M - 1);
        bm = min(max(bm, 0), M - 1);
        bn = min(max(bn, 0), N - 1);
        const int kind = (g >= 2) ? 1 : P.bc_kind[side];
        const bool zside = side < 2;
        R v[4];
        if (kind == 0) {            // REFLECT
            const int si = mn - n0 + 2 + QX, sj = mm - m0 + 2;
            v[0] = q[0][sj][si]; v[1] = q[1][sj][si]; v[2] = q[2][sj][si]; v[3] = q[3][sj][si];
            if (zside) v[2] = -v[2]; else v[3] = -v[3];
        } else if (kind == 2) {     // FIXED
            v[0] = (R)P.bc_val[side][0]; v[1] = (R)P.bc_val[side][1];
            v[2] = (R)P.bc_val[side][2]; v[3] = (R)P.bc_val[side][3];
        } else {                    // OUTFLOW, SUCTION, NONREFLECT, deeper ghost layers
            const int si = bn - n0 + 2 + QX, sj = bm - m0 + 2;
            v[0] = q[0][sj][si]; v[1] = q[1][sj][si]; v[2] = q[2][sj][si]; v[3] = q[3][sj][si];
            if (kind == 3) {
                ghost_suction(zside, low, (R)(zside ? P.bc_val[side][2] : P.bc_val[side][3]), v);
            } else if (kind == 4) {
                ghost_nonreflect(gas_of<R>(P), zside, low, v);
            }
        }
        q[0][j][i + QX] = v[0]; q[1][j][i + QX] = v[1]; q[2][j][i + QX] = v[2]; q[3][j][i + QX] = v[3];
    }
}

// The FP64 kernels call it out of line (a smaller persistent kernel: the
// wind problem, whose fixed region sends every tile through here, 1.512 ->
// 1.480 ms per step in FP64); the FP32 kernels inline it (out of line the
// call's register saves cost them 4-8%).
template <typename R, int TZ, int TR, typename S>
__device__ __noinline__ void patch_tile_out(const StepParams& P, S& sm, int b, int n0, int m0)
{
    patch_tile_body<R, TZ, TR>(P, sm, b, n0, m0);
}
template <typename R, int TZ, int TR, typename S>
__device__ __forceinline__ void patch_tile(const StepParams& P, S& sm, int b, int n0, int m0)
{
    if constexpr (sizeof(R) == 8) patch_tile_out<R, TZ, TR>(P, sm, b, n0, m0);
    else patch_tile_body<R, TZ, TR>(P, sm, b, n0, m0);
}

// The wave speed and flux of a face whose two sides hold the state
// (r, p, un, ut) (face frame), as face_flux finds them for identical states
// in the high-order region: the exact solver's identical-state branch, the
// HLL-family functions themselves.
template <typename R, int FLUX>
__device__ __forceinline__ R uniform_face(const Gas<R>& g, R r, R p, R un, R ut, R F[4])
{
    if constexpr (FLUX == 2) {
        const R cs = sqrt(g.ga * p / r);
        const R m = r * un;
        F[0] = m;
        F[1] = m * un + p;
        F[2] = m * ut;
        F[3] = un * (p * g.inv_g1 + R(0.5) * r * (un * un + ut * ut) + p);
        return fmax(fabs(un) + cs, g.eps8);
    } else if constexpr (FLUX == 1) {
        return flux_hllc(g, r, p, un, ut, r, p, un, ut, F);
    } else if constexpr (FLUX == 3) {
        return flux_hllc_a(g, r, p, un, ut, r, p, un, ut, F);
    } else if constexpr (FLUX == 4) {
        R FQ;
        return flux_hllcq(g, r, p, un, ut, R(0), r, p, un, ut, R(0), F, FQ);
    } else {
        return flux_hll(g, r, p, un, ut, r, p, un, ut, F);
    }
}

// A uniform tile (skip_uniform): every staged cell a face of the tile reads
// (the tile's rows over the full halo width, its columns over the full halo
// height, ghost cells included) holds the bits of tile cell (0, 0), and the
// flux of that state is finite.  Then every face of one orientation has the
// same flux, the update's flux differences are exactly zero, and only the
// wave speeds of the two orientations are needed: returned in sz / sr
// (valid in thread 0).  A barrier: called by all threads.
template <typename R, int FLUX, int TZ, int TR, typename S>
__device__ __forceinline__ bool tile_uniform(const S& sm, int b, const Gas<R>& g, R& sz, R& sr)
{
    constexpr int HZ = S::HZ, HR = S::HR, QX = S::QX;
    using U = std::conditional_t<sizeof(R) == 4, unsigned int, unsigned long long>;
    const auto& q = sm.qb[b];
    auto bits = [](R v) { return *reinterpret_cast<const U*>(&v); };
    const R s0 = q[0][2][2 + QX], s1 = q[1][2][2 + QX], s2 = q[2][2][2 + QX], s3 = q[3][2][2 + QX];
    const U r0 = bits(s0), r1 = bits(s1), r2 = bits(s2), r3 = bits(s3);
    bool same = true;
    for (int idx = threadIdx.x; idx < HR * HZ; idx += kThreads) {
        const int j = idx / HZ, i = idx - j * HZ;
        const bool rin = (j >= 2 && j < TR + 2), cin = (i >= 2 && i < TZ + 2);
        if (!rin && !cin) continue;   // the corners: read by no face
        same = same && bits(q[0][j][i + QX]) == r0 && bits(q[1][j][i + QX]) == r1 && bits(q[2][j][i + QX]) == r2 &&
               bits(q[3][j][i + QX]) == r3;
    }
    if (threadIdx.x == 0) {
        R F[4], G[4];
        sz = uniform_face<R, FLUX>(g, s0, s1, s2, s3, F);   // z faces: normal v_z
        sr = uniform_face<R, FLUX>(g, s0, s1, s3, s2, G);   // r faces: normal v_r
        for (int k = 0; k < 4; k++) same = same && isfinite(F[k]) && isfinite(G[k]);
        same = same && isfinite(sz) && isfinite(sr);
    }
    return __syncthreads_and(same);
}

// faces, exact-solver queue and conservative update of the tile staged in
// buffer b.  TO_SMEM: the updated cells go to sm.out (for a bulk store)
// instead of global memory.  Ends without a barrier.
template <typename R, int FLUX, bool RECON, int LAYOUT, int TZ, int TR, bool TO_SMEM, bool SKIP = true,
          bool LATE_K = false, typename S>
__device__ __forceinline__ void tile_body(const StepParams& P, S& sm, int b, const Gas<R>& g, int n0, int m0,
                                          const StepConsts& K, TileAcc<R>& acc)
{
    constexpr int QX = S::QX;
    // ---- every face of the tile once, then the queue
    // r of the tile's rows for the update (the barrier after the faces
    // orders these writes before their use)
    if (threadIdx.x < TR) {
        const int m = m0 + threadIdx.x;
        const double yd = P.y_min + m * P.dy;
        const float yf = P.y_minf + (float)m * P.dyf;
        sm.ydrow[threadIdx.x] = yd;
        sm.yfrow[threadIdx.x] = yf;
        // FP64 kernels: the axisymmetric source's T_do / r once per row, not
        // once per cell (the same expression, the same values).  Not in
        // FP32: there the division per cell is a reciprocal and a multiply,
        // cheaper than an FP64 division at every tile's start, and the FP32
        // persistent batch kernel sets K only during the face pass.
        if constexpr (sizeof(R) == 8) sm.tydrow[threadIdx.x] = (P.geom == 1) ? K.T_do / yd : 0.0;
        if constexpr (sizeof(R) == 4 && !LATE_K) sm.tyfrow[threadIdx.x] = (P.geom == 1) ? K.T_f / yf : 0.0f;
    }
    // SKIP: the kernel carries the uniform-tile test (skip_uniform); the
    // persistent kernel has a variant without it, so that the default path
    // holds none of its code
    bool skipped = false;
    R sz, sr;
    if (SKIP && P.skip_uniform && !P.region_select && !tile_near_fixed<TZ, TR>(P, n0, m0) &&
        tile_uniform<R, FLUX, TZ, TR>(sm, b, g, sz, sr)) {
        skipped = true;
        // zero fluxes (the same flux on every face of an orientation: its
        // differences are exactly zero) and the two wave speeds
        constexpr int NF4 = (TR * (TZ + 1) + (TR + 1) * TZ) * 4;
        R* fz = &sm.Fz[0][0][0];
        R* fr = &sm.Fr[0][0][0];
        for (int w = threadIdx.x; w < NF4 / 4; w += kThreads) {
            R* d = (w < TR * (TZ + 1)) ? fz + 4 * w : fr + 4 * (w - TR * (TZ + 1));
            put4(d, R(0), R(0), R(0), R(0));
        }
        if (threadIdx.x == 0) {
            acc.smz = fmax(acc.smz, sz);
            acc.smr = fmax(acc.smr, sr);
        }
    }
    if (!skipped)
        face_pass<R, FLUX, RECON, TZ, TR, SKIP>(P, sm, b, g, n0, m0, K.step, acc.rc, acc.fallback, acc.smz, acc.smr);
    // persistent kernel: the previous tile's bulk store, issued by the copy
    // thread at the start of this face pass, has read sm.out before anything
    // overwrites it (the network's space in the queue phase, then the update)
    if constexpr (TO_SMEM) {
        if (threadIdx.x == kCopyThread) tma::store_wait_read();
    }
    __syncthreads();
    phase_mark(2);
    if constexpr (FLUX == 2) {
        queue_pass<R, RECON, TZ, TR>(P, sm, b, g, n0, m0, K.step, acc.rc, acc.fallback, acc.smz, acc.smr);
        __syncthreads();
        phase_mark(3);
        // persistent kernels: the next tile's queue starts empty (ordered
        // before its face pass by the barrier between the tiles)
        if constexpr (TO_SMEM) {
            if (threadIdx.x == kCopyThread) sm.qn = 0u;
        }
    }

    // ---- conservative update of the tile's cells
    const float tdv_f = K.tdv_f, Tf = K.T_f, dxf = P.dxf, dyf = P.dyf;
    const float gaf = P.gf.ga, g1f = P.gf.g1, ig1f = P.gf.inv_g1;
    const auto& qv = sm.qb[b];
    // cell cidx of the tile: its staged state and its four face fluxes
    auto load_cell = [&](int row, int col, R in[4], R f[4][4]) {
        const int j = row + 2, i = col + 2;
        in[0] = qv[0][j][i + QX]; in[1] = qv[1][j][i + QX]; in[2] = qv[2][j][i + QX]; in[3] = qv[3][j][i + QX];
        get4(sm.Fz[row][col + 1], f[0][0], f[1][0], f[2][0], f[3][0]);
        get4(sm.Fz[row][col], f[0][1], f[1][1], f[2][1], f[3][1]);
        get4(sm.Fr[row][col], f[0][2], f[1][2], f[2][2], f[3][2]);
        get4(sm.Fr[row + 1][col], f[0][3], f[1][3], f[2][3], f[3][3]);
    };
    // the update in FP64 (the FP64 solver; in the FP32 form the four cell
    // rows next to the axis, where the 1/r source is largest); the step's
    // FP64 constants read where they are used (not held in registers
    // through the FP32 form's loop)
    auto update_fp64 = [&](int row, int n, const R in[4], const R f[4][4], R o[4]) {
        const double T_do = K.T_do, tdv_d = K.tdv;
        const double y = sm.ydrow[row];
        double Q2 = 0.0, Sz = 0.0, Sr = 0.0;
        if (P.body_force) {
            const double x = P.x_min + n * P.dx;
            if (x > P.body_lo && x < P.body_hi)
                Q2 = (y >= P.body_rsplit) ? -P.body_amp * (double)in[0] : P.body_amp * (double)in[0];
        }
        // the neutral-coupling source in the update (FP64 kernels; the FP32
        // form adds it in neutral_kernel after the step)
        if (sizeof(R) == 8 && P.nsrc) {
            double az, ar;
            neutral_at<R, LAYOUT, TO_SMEM>(P, n, m0 + row, az, ar);
            const double w = T_do * ((double)in[0] * P.nsrc_coef);
            Sz = w * az;
            Sr = w * ar;
        }
        const double ty = (sizeof(R) == 8) ? sm.tydrow[row] : ((P.geom == 1) ? T_do / y : 0.0);
        update_cell<double>(P, P.gd.ga, P.gd.g1, P.gd.inv_g1, in, f, T_do, tdv_d, ty, P.dx, P.dy, Q2, Sz, Sr,
                            acc.nrho, acc.np, acc.rc.status, o);
    };
    // the FP32 form's source terms of a cell: ty = T_do/r and the body force
    auto sources_fp32 = [&](int row, int n, const R in[4], float& ty, float& Q2) {
        const float y = sm.yfrow[row];
        Q2 = 0.0f;
        if (P.body_force) {
            const float x = P.x_minf + (float)n * dxf;
            if (x > P.body_lof && x < P.body_hif)
                Q2 = (y >= P.body_rsplitf) ? -P.body_ampf * (float)in[0] : P.body_ampf * (float)in[0];
        }
        if constexpr (LATE_K) ty = (P.geom == 1) ? Tf / y : 0.0f;
        else ty = sm.tyfrow[row];
    };
    auto store_cell = [&](int row, int col, int n, int m, const R o[4], bool p_only) {
        if constexpr (TO_SMEM) {
            sm.out[1][row][col] = o[1];
            if (!p_only) { sm.out[0][row][col] = o[0]; sm.out[2][row][col] = o[2]; sm.out[3][row][col] = o[3]; }
        } else if (LAYOUT == kSoA) {
            R* out = (R*)P.out;
            const long long k = (long long)m * P.ld + n;
            out[k + P.plane] = o[1];
            if (!p_only) { out[k] = o[0]; out[k + 2 * P.plane] = o[2]; out[k + 3 * P.plane] = o[3]; }
        } else {
            const long long k = (long long)m * P.N + n;
            ((double2*)P.out)[k] = make_double2((double)o[0], (double)o[1]);
            if (!p_only) ((double2*)P.out_u)[k] = make_double2((double)o[2], (double)o[3]);
        }
    };
    // FP32 form: cells whose FP64 part is done after the loop, so that its
    // code stays out of the loop's register allocation (bit 2 it: a
    // near-axis cell, its whole update; bit 2 it + 1: the FP64 pressure
    // recovery of a cell whose kinetic energy is above 99% of the total)
    unsigned deferred = 0u;
    // a fixed number of cells per thread (the loop unrolls; the uniform
    // tests and the index arithmetic are shared by the thread's cells)
    static_assert((TZ * TR) % kThreads == 0, "whole cells per thread");
#pragma unroll
    for (int it = 0; it < (TZ * TR) / kThreads; it++) {
        const int cidx = (int)threadIdx.x + it * kThreads;
        const int row = cidx / TZ, col = cidx - row * TZ;
        const int n = n0 + col, m = m0 + row;
        if (n >= P.N || m >= P.M) continue;
        const int j = row + 2, i = col + 2;
        R o[4] = {qv[0][j][i + QX], qv[1][j][i + QX], qv[2][j][i + QX], qv[3][j][i + QX]};
        if (!(P.fixed_region && sm.fx[j][i])) {
            R in[4], f[4][4];
            load_cell(row, col, in, f);
            if constexpr (sizeof(R) == 8) {
                update_fp64(row, n, in, f, o);
            } else {
                if (P.geom == 1 && m < 4) {
                    deferred |= 1u << (2 * it);
                    continue;
                }
                float ty, Q2;
                sources_fp32(row, n, in, ty, Q2);
                float E2, KE2;
                update_cell<float>(P, gaf, g1f, ig1f, in, f, Tf, tdv_f, ty, dxf, dyf, Q2, 0.0f, 0.0f, acc.nrho, acc.np,
                                   acc.rc.status, o, &E2, &KE2);
                // pressure recovery p = (g-1)(E - rho v^2/2) in FP64 where
                // the kinetic energy is more than 99% of the total
                if (KE2 > 0.99f * E2) deferred |= 2u << (2 * it);
            }
        }
        store_cell(row, col, n, m, o, false);
    }
    if constexpr (sizeof(R) == 4) {
        static_assert(TO_SMEM || LAYOUT == kSoA, "FP32 state is SoA planes");
        if (deferred) {
            for (int it = 0; it < (TZ * TR) / kThreads; it++) {
                const int cidx = (int)threadIdx.x + it * kThreads;
                const unsigned d = (deferred >> (2 * it)) & 3u;
                if (!d) continue;
                const int row = cidx / TZ, col = cidx - row * TZ;
                const int n = n0 + col, m = m0 + row;
                R in[4], f[4][4], o[4];
                load_cell(row, col, in, f);
                if (d & 1u) {
                    update_fp64(row, n, in, f, o);
                    store_cell(row, col, n, m, o, false);
                } else {
                    float ty, Q2;
                    sources_fp32(row, n, in, ty, Q2);
                    o[1] = (R)pressure_fp64(P, in, f, tdv_f, ty, Tf, Q2, dxf, dyf, acc.np);
                    store_cell(row, col, n, m, o, true);
                }
            }
        }
    }
    phase_mark(4);
}

// Block reduction of the CTA's accumulators and the step epilogue.  `units`
// = the number of tickets of this problem and step (`weight` tickets per
// report: one per CTA, or one per tile for a report covering several
// tiles); the last reporter turns the wave-speed maxima into the next dt and
// performs the reference's funk_time shift (kernel.cu:1525-1536), and with
// reset_tiles also rewinds the tile counter of the persistent kernel.
template <typename R>
__device__ __forceinline__ void cta_epilogue(const StepParams& P, TileAcc<R>& acc, unsigned int units,
                                             bool reset_tiles, unsigned int weight = 1u)
{
    __shared__ R red_r[2][kThreads / 32];
    __shared__ int red_i[4][kThreads / 32];
    __shared__ int s_last;
    const int tid = threadIdx.x;
    const int lane = tid & 31, wid = tid >> 5;
    RiemannCount& rc = acc.rc;
    {
        const R a = warp_max(acc.smz), b = warp_max(acc.smr);
        const int c0 = __reduce_add_sync(0xffffffffu, acc.nrho), c1 = __reduce_add_sync(0xffffffffu, acc.np);
        const int c2 = __reduce_add_sync(0xffffffffu, acc.fallback);
        const unsigned st = __reduce_or_sync(0xffffffffu, rc.status);
        if (lane == 0) {
            red_r[0][wid] = a; red_r[1][wid] = b;
            red_i[0][wid] = c0; red_i[1][wid] = c1; red_i[2][wid] = (int)st; red_i[3][wid] = c2;
        }
        if (P.collect_stats && P.clock != nullptr) {
            const int n1 = __reduce_add_sync(0xffffffffu, rc.newton_calls);
            const int n2 = __reduce_add_sync(0xffffffffu, rc.newton_iters);
            const int b1 = __reduce_add_sync(0xffffffffu, rc.bisect_calls);
            const int b2 = __reduce_add_sync(0xffffffffu, rc.bisect_iters);
            const unsigned nm = __reduce_max_sync(0xffffffffu, (unsigned)rc.newton_max);
            const int s1 = __reduce_add_sync(0xffffffffu, rc.strong_calls);
            const int s2 = __reduce_add_sync(0xffffffffu, rc.strong_iters);
            if (lane == 0) {
                if (s1) atomicAdd(&P.clock->cnt[8], (unsigned long long)s1);
                if (s2) atomicAdd(&P.clock->cnt[9], (unsigned long long)s2);
                if (n1) atomicAdd(&P.clock->cnt[2], (unsigned long long)n1);
                if (n2) atomicAdd(&P.clock->cnt[3], (unsigned long long)n2);
                if (b1) atomicAdd(&P.clock->cnt[4], (unsigned long long)b1);
                if (b2) atomicAdd(&P.clock->cnt[5], (unsigned long long)b2);
                if (nm) atomicMax(&P.clock->cnt[7], (unsigned long long)nm);
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        R ar = R(0), br = R(0);
        int c0 = 0, c1 = 0, c2 = 0;
        unsigned st = 0;
        for (int w = 0; w < kThreads / 32; w++) {
            ar = fmax(ar, red_r[0][w]); br = fmax(br, red_r[1][w]);
            c0 += red_i[0][w]; c1 += red_i[1][w]; st |= (unsigned)red_i[2][w]; c2 += red_i[3][w];
        }
        if (c0) st |= 0x01u;
        if (c1) st |= 0x02u;
        if (c2) st |= 0x40u;
        const double a = (double)ar, b = (double)br;
        if (P.clock != nullptr) {
            DevClock* C = P.clock;
            if (a > 0.0) atomicMax(&C->smax_z, (unsigned long long)__double_as_longlong(a));
            if (b > 0.0) atomicMax(&C->smax_r, (unsigned long long)__double_as_longlong(b));
            if (c0) atomicAdd(&C->cnt[0], (unsigned long long)c0);
            if (c1) atomicAdd(&C->cnt[1], (unsigned long long)c1);
            if (c2) atomicAdd(&C->cnt[6], (unsigned long long)c2);
            if (st) atomicOr(&C->status, st);
            __threadfence();
            const unsigned int ticket = atomicAdd(&C->done, weight);
            s_last = (ticket + weight == units) ? 1 : 0;
        } else {
            // raw mode: this CTA's dt candidate, min-reduced into *T_min
            double dt = P.dt_cap;
            if (a > 0.0) dt = fmin(dt, P.krit_dx / a);
            if (b > 0.0) dt = fmin(dt, P.krit_dy / b);
            atomicMin((unsigned long long*)P.T_min, (unsigned long long)__double_as_longlong(dt));
            if (st && P.status_ptr) atomicOr(P.status_ptr, st);
            s_last = 0;
        }
    }
    __syncthreads();
    if (s_last && tid == 0) {
        // funk_time (kernel.cu:1525-1536): T_do <- min dt, TT += T_do, i++
        __threadfence();
        DevClock* C = P.clock;
        const double a = __longlong_as_double((long long)atomicExch(&C->smax_z, 0ull));
        const double b = __longlong_as_double((long long)atomicExch(&C->smax_r, 0ull));
        double dt = P.dt_cap;
        if (a > 0.0) dt = fmin(dt, P.krit_dx / a);
        if (b > 0.0) dt = fmin(dt, P.krit_dy / b);
        C->T_prev = C->T_do;
        C->T_do = dt;
        C->TT = C->TT + dt;
        C->step = C->step + 1;
        C->done = 0u;
        if (reset_tiles) C->next_tile = 0u;
        __threadfence();
    }
}

// Tile (bx, by) of the problem P; `tiles` is the number of tiles of that
// problem (the last of them to finish performs the dt epilogue).
template <typename R, int FLUX, bool RECON, int LAYOUT, int TZ, int TR>
__device__ __forceinline__ void step_tile(const StepParams& P, int bx, int by, unsigned int tiles)
{
    using S = TileSmem<R, FLUX, TZ, TR>;
    S& sm = tile_smem<S>();
    __shared__ StepConsts sK;
    const int n0 = bx * TZ, m0 = by * TR;
    const Gas<R>& g = *reinterpret_cast<const Gas<R>*>(sizeof(R) == 8 ? (const void*)&P.gd : (const void*)&P.gf);
    if (threadIdx.x == 0) {
        sm.qn = 0u;
        step_consts(P, sK);
    }
    stage_tile<R, LAYOUT, TZ, TR>(P, sm, 0, n0, m0);
    __syncthreads();
    TileAcc<R> acc;
    acc.clear();
    tile_body<R, FLUX, RECON, LAYOUT, TZ, TR, false>(P, sm, 0, g, n0, m0, sK, acc);
    cta_epilogue<R>(P, acc, tiles, false);
}

// ------------------------------------------------------------------ the kernels
// CTAs per SM the register allocation is sized for: FP64 2 (shared memory
// allows no more); FP32 4 (64 registers; the exact solver spills a few
// dozen bytes there and still runs 13% faster than at 3 CTAs and 85
// registers, measured at 4096x2048)
template <typename R, int FLUX>
constexpr int min_ctas() { return sizeof(R) == 8 ? 2 : 4; }

// one problem: a CTA per tile, grid (tiles along z, tiles along r)
template <typename R, int FLUX, bool RECON, int LAYOUT, int TZ, int TR>
__global__ void __launch_bounds__(kThreads, min_ctas<R, FLUX>()) step_kernel(StepParams P)
{
    step_tile<R, FLUX, RECON, LAYOUT, TZ, TR>(P, blockIdx.x, blockIdx.y + P.band_lo,
                                              P.units > 0 ? (unsigned)P.units : gridDim.x * gridDim.y);
}

// many problems of one (flux, recon) class: a CTA per (problem, tile) of the
// work list.  Problem j of the class owns CTAs tile_start[j] ..
// tile_start[j+1]-1, its tiles in row-major order; its parameters are
// Ps[j] (copied into shared memory once per CTA).
template <typename R, int FLUX, bool RECON, int TZ, int TR>
__global__ void __launch_bounds__(kThreads, min_ctas<R, FLUX>())
    batch_kernel(const StepParams* __restrict__ Ps, const int* __restrict__ tile_start, int nprob)
{
    __shared__ __align__(16) StepParams sP;
    __shared__ int s_j;
    if (threadIdx.x == 0) {
        // the last problem whose first tile is at or before this CTA
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tile_start[mid] <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
        }
        s_j = lo;
    }
    __syncthreads();
    const int j = s_j;
    static_assert(sizeof(StepParams) % 16 == 0, "StepParams is copied as 16-byte words");
    for (int w = threadIdx.x; w < (int)(sizeof(StepParams) / 16); w += kThreads)
        reinterpret_cast<int4*>(&sP)[w] = reinterpret_cast<const int4*>(Ps + j)[w];
    __syncthreads();
    const int t = (int)blockIdx.x - tile_start[j];
    const int tz = (sP.N + TZ - 1) / TZ;
    step_tile<R, FLUX, RECON, kSoA, TZ, TR>(sP, t % tz, t / tz, (unsigned)(tile_start[j + 1] - tile_start[j]));
}

// Many problems of any fluxes (one reconstruction) in one launch: as
// batch_kernel, each CTA then steps its tile with the tile code of its
// problem's flux, flux_of[j] = the kernels' FLUX (0 HLL, 1 HLLC, 2 exact
// Godunov, 3 HLLC_Aleksashov); a CTA runs one of the four, and the dynamic
// shared memory is the largest of their tile spaces
template <typename R, bool RECON, int TZ, int TR>
__global__ void __launch_bounds__(kThreads, min_ctas<R, 2>())
    batch_kernel_mixed(const StepParams* __restrict__ Ps, const int* __restrict__ tile_start,
                       const int* __restrict__ flux_of, int nprob)
{
    __shared__ __align__(16) StepParams sP;
    __shared__ int s_j;
    if (threadIdx.x == 0) {
        int lo = 0, hi = nprob - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (tile_start[mid] <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
        }
        s_j = lo;
    }
    __syncthreads();
    const int j = s_j;
    for (int w = threadIdx.x; w < (int)(sizeof(StepParams) / 16); w += kThreads)
        reinterpret_cast<int4*>(&sP)[w] = reinterpret_cast<const int4*>(Ps + j)[w];
    __syncthreads();
    const int t = (int)blockIdx.x - tile_start[j];
    const int tz = (sP.N + TZ - 1) / TZ;
    const unsigned tiles = (unsigned)(tile_start[j + 1] - tile_start[j]);
    switch (flux_of[j]) {
    case 0: step_tile<R, 0, RECON, kSoA, TZ, TR>(sP, t % tz, t / tz, tiles); break;
    case 1: step_tile<R, 1, RECON, kSoA, TZ, TR>(sP, t % tz, t / tz, tiles); break;
    case 3: step_tile<R, 3, RECON, kSoA, TZ, TR>(sP, t % tz, t / tz, tiles); break;
    default: step_tile<R, 2, RECON, kSoA, TZ, TR>(sP, t % tz, t / tz, tiles); break;
    }
}

// The FP32 solver's persistent kernel: as many CTAs as fit on the GPU at
// once, each taking tiles from a counter in the clock until none are left.
// A tile and its halo arrive by one bulk-tensor copy of the box (x = z
// cells n0-4 .. n0+TZ+3, y = rows m0-2 .. m0+TR+1, all four planes) into
// one of two buffers; the copy of the CTA's next tile runs while the current
// one is computed.  The updated cells leave by a bulk-tensor store from a
// shared-memory tile.  The bulk copies, the store and the counter's atomic
// are issued by one thread of the last warp at the start of the face pass
// (their issue takes hundreds of cycles; that warp has one face fewer to
// compute than the first two, so the barrier after the faces does not wait
// for it): the store of the previous tile's cells, the copy of the next
// tile, and the counter's atomic for the tile after it.  The CTA's
// wave-speed maxima and counters accumulate over its tiles and are reported
// once (one ticket per CTA).  A bulk copy that does not arrive within the
// wait limit (P.wait_polls) sets AST_ST_TIMEOUT and is waited for with the
// long limit; one that does not arrive even then ends the CTA's loop.
template <typename R, int FLUX, bool RECON, bool SKIP>
__global__ void __launch_bounds__(kThreads, sizeof(R) == 4 ? 4 : 2)
    step_kernel_tma(StepParams P, const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout)
{
    constexpr int TZ = kTmaTZ, TR = kTmaTR;
    using S = TileSmem<R, FLUX, TZ, TR, 2>;
    constexpr uint32_t kBoxBytes = 4u * S::HR * S::HZP * sizeof(R);
    static_assert(sizeof(((S*)nullptr)->qb[0]) == kBoxBytes, "tile buffer is the TMA box");
    S& sm = tile_smem<S>();
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int s_tile[2];      // tiles of the current and the next iteration (per buffer)
    __shared__ int2 s_org[2];      // their origins (n0, m0), set with s_tile by the copy thread
    __shared__ StepConsts sK;
    __shared__ int2 s_pend;        // copy thread: origin of the tile whose cells wait in sm.out
    const int tid = threadIdx.x;
    const bool copier = tid == kCopyThread;
    const int tiles_z = (P.N + TZ - 1) / TZ;
    const int t_lo = P.band_lo * tiles_z;   // this launch's tiles: t_lo <= t < tiles
    const int tiles = tiles_z * (P.band_hi > 0 ? P.band_hi : (P.M + TR - 1) / TR);
    if (copier) {
        tma::prefetch_map(&tin);
        tma::prefetch_map(&tout);
        tma::mbar_init(&bar[0], 1);
        tma::mbar_init(&bar[1], 1);
        tma::fence_async_shared();
        step_consts(P, sK);
        s_pend = make_int2(-1, -1);
        sm.qn = 0u;   // later tiles: reset after the previous tile's queue
        // the first two tiles: the first is copied now, the second at the
        // start of the first tile's face pass
        const int t0 = t_lo + (int)atomicAdd(&P.clock->next_tile, 1u);
        const int t1 = (t0 < tiles) ? t_lo + (int)atomicAdd(&P.clock->next_tile, 1u) : tiles;
        s_tile[0] = t0;
        s_tile[1] = t1;
        s_org[1] = make_int2((t1 % tiles_z) * TZ, (t1 / tiles_z) * TR);
        if (t0 < tiles) {
            s_org[0] = make_int2((t0 % tiles_z) * TZ, (t0 / tiles_z) * TR);
            tma::mbar_expect(&bar[0], kBoxBytes);
            tma::load_3d(&tin, &sm.qb[0][0][0][0], &bar[0], s_org[0].x - 4, s_org[0].y - 2, 0);
        }
    }
    __syncthreads();
    phase_mark(kPhaseStart);
    TileAcc<R> acc;
    acc.clear();
    const Gas<R>& g = gas_of<R>(P);
    for (int k = 0;; k++) {
        const int b = k & 1;
        const int t = s_tile[b];
        if (t >= tiles) break;
        // the origin the copy thread found (one integer division per tile,
        // not one per thread), read before the barrier below, after which
        // the copy thread overwrites this buffer's slots
        const int n0 = s_org[b].x, m0 = s_org[b].y;
        // The barrier after the copy's arrival is the one barrier between
        // two tiles: every thread has finished the previous tile (its
        // update and its reads of the other buffer and of the output tile)
        // and fenced its shared-memory writes for the bulk copies.
        bool arrived = tma::mbar_wait(&bar[b], (uint32_t)((k >> 1) & 1), P.wait_polls);
        if (__syncthreads_or(!arrived)) {
            // the copy did not arrive within the wait limit: reported, then
            // waited for with the long limit (every CTA leaves with no copy
            // in flight; the next tile's copy is not issued yet), and the
            // tile is computed when it has arrived.  A copy that does not
            // arrive even then ends this CTA's tiles.
            if (copier) acc.rc.status |= AST_ST_TIMEOUT;
            arrived = tma::mbar_wait(&bar[b], (uint32_t)((k >> 1) & 1));
            if (__syncthreads_or(!arrived)) break;
        }
        phase_mark(0);
        // ghost cells (tiles at the grid's edge or near the fixed region
        // only: the others need no second barrier)
        if (n0 - 2 < 0 || n0 + TZ + 2 > P.N || m0 - 2 < 0 || m0 + TR + 2 > P.M || P.fixed_region) {
            patch_tile<R, TZ, TR>(P, sm, b, n0, m0);
            __syncthreads();
        }
        phase_mark(1);
        if (copier) {
            // the previous tile's cells (sm.out is not written again before
            // the store has read it: see tile_body)
            const int2 pend = s_pend;
            if (pend.x >= 0) {
                tma::store_3d(&tout, &sm.out[0][0][0], pend.x, pend.y, 0);
                tma::store_commit();
            }
            s_pend = make_int2(n0, m0);
            // the next tile's box into the other buffer (last read by the
            // previous tile, which every thread finished before the barriers
            // above), then the counter's atomic for the tile after it, into
            // this buffer's slots (every thread has read them)
            int tnn = tiles;
            if (s_tile[b ^ 1] < tiles) {
                tma::mbar_expect(&bar[b ^ 1], kBoxBytes);
                tma::load_3d(&tin, &sm.qb[b ^ 1][0][0][0], &bar[b ^ 1], s_org[b ^ 1].x - 4, s_org[b ^ 1].y - 2,
                             0);
                tnn = t_lo + (int)atomicAdd(&P.clock->next_tile, 1u);
            }
            s_tile[b] = tnn;
            s_org[b] = make_int2((tnn % tiles_z) * TZ, (tnn / tiles_z) * TR);
        }
        tile_body<R, FLUX, RECON, kSoA, TZ, TR, true, SKIP>(P, sm, b, g, n0, m0, sK, acc);
        // this thread's shared-memory writes (sm.out, ghost cells) before
        // the bulk copies that read or overwrite them (ordered by the next
        // tile's barrier, or the one below)
        tma::fence_async_shared();
    }
    __syncthreads();
    if (copier) {
        const int2 pend = s_pend;
        if (pend.x >= 0) {
            tma::store_3d(&tout, &sm.out[0][0][0], pend.x, pend.y, 0);
            tma::store_commit();
        }
        tma::store_wait_all();
    }
    cta_epilogue<R>(P, acc, P.units > 0 ? (unsigned)P.units : gridDim.x, true);
    phase_mark(5);
    phase_mark(kPhaseFlush, P.clock);
}

// A tile of the persistent batch kernels' work list: its problem's slot and
// tile code (slot | FLUX << 24), origin and clock.
struct __align__(16) BatchTile {
    int sf;
    int n0, m0;
    int rsv_;
    DevClock* clock;
    long long rsv2_;
};
static_assert(sizeof(BatchTile) == 32, "a work-list entry is two 16-byte copies");

// One run of consecutive tiles of one problem, reported by every warp
// without a barrier: the warp's wave-speed maxima (atomic maxima on the
// clock), floor and fallback counts, status bits and solver counters.
template <typename R>
__device__ __forceinline__ void warp_report(const StepParams& P, const TileAcc<R>& acc)
{
    DevClock* C = P.clock;
    const R a = warp_max(acc.smz), b = warp_max(acc.smr);
    const int c0 = __reduce_add_sync(0xffffffffu, acc.nrho), c1 = __reduce_add_sync(0xffffffffu, acc.np);
    const int c2 = __reduce_add_sync(0xffffffffu, acc.fallback);
    unsigned st = __reduce_or_sync(0xffffffffu, acc.rc.status);
    const RiemannCount& rc = acc.rc;
    int n1 = 0, n2 = 0, b1 = 0, b2 = 0, s1 = 0, s2 = 0;
    unsigned nm = 0;
    if (P.collect_stats) {
        n1 = __reduce_add_sync(0xffffffffu, rc.newton_calls);
        n2 = __reduce_add_sync(0xffffffffu, rc.newton_iters);
        b1 = __reduce_add_sync(0xffffffffu, rc.bisect_calls);
        b2 = __reduce_add_sync(0xffffffffu, rc.bisect_iters);
        nm = __reduce_max_sync(0xffffffffu, (unsigned)rc.newton_max);
        s1 = __reduce_add_sync(0xffffffffu, rc.strong_calls);
        s2 = __reduce_add_sync(0xffffffffu, rc.strong_iters);
    }
    if ((threadIdx.x & 31) == 0) {
        if (c0) st |= 0x01u;
        if (c1) st |= 0x02u;
        if (c2) st |= 0x40u;
        const double da = (double)a, db = (double)b;
        if (da > 0.0) atomicMax(&C->smax_z, (unsigned long long)__double_as_longlong(da));
        if (db > 0.0) atomicMax(&C->smax_r, (unsigned long long)__double_as_longlong(db));
        if (c0) atomicAdd(&C->cnt[0], (unsigned long long)c0);
        if (c1) atomicAdd(&C->cnt[1], (unsigned long long)c1);
        if (c2) atomicAdd(&C->cnt[6], (unsigned long long)c2);
        if (st) atomicOr(&C->status, st);
        if (n1) atomicAdd(&C->cnt[2], (unsigned long long)n1);
        if (n2) atomicAdd(&C->cnt[3], (unsigned long long)n2);
        if (b1) atomicAdd(&C->cnt[4], (unsigned long long)b1);
        if (b2) atomicAdd(&C->cnt[5], (unsigned long long)b2);
        if (nm) atomicMax(&C->cnt[7], (unsigned long long)nm);
        if (s1) atomicAdd(&C->cnt[8], (unsigned long long)s1);
        if (s2) atomicAdd(&C->cnt[9], (unsigned long long)s2);
    }
}

// funk_time (kernel.cu:1525-1536) of one problem after every tile of its
// step has reported: T_do <- min dt, TT += T_do, step + 1
__device__ __forceinline__ void clock_shift(const StepParams& P)
{
    DevClock* C = P.clock;
    const double a = __longlong_as_double((long long)atomicExch(&C->smax_z, 0ull));
    const double b = __longlong_as_double((long long)atomicExch(&C->smax_r, 0ull));
    double dt = P.dt_cap;
    if (a > 0.0) dt = fmin(dt, P.krit_dx / a);
    if (b > 0.0) dt = fmin(dt, P.krit_dy / b);
    C->T_prev = C->T_do;
    C->T_do = dt;
    C->TT = C->TT + dt;
    C->step = C->step + 1;
    C->done = 0u;
}

// The persistent FP32 batch kernel: the tiles of many problems handed out by
// one counter over a work list (`work`: every problem's 32x16 tiles in
// row-major order, the problems in slot order).  One class of problems
// (MIXED false: every tile has the kernel's FLUX), or every problem of the
// batch in one launch (MIXED true: each tile is stepped with the tile code of
// its own FLUX, all in the exact solver's shared-memory layout).
//
// The copy thread stages the next tile's box by a bulk-tensor copy through
// its problem's tensor map together with the problem's parameters (a bulk
// copy of its StepParams) on the buffer's mbarrier, fetches that tile's dt
// and step from its clock and the work-list entry of the tile after it
// (asynchronous copies into shared memory) and claims that tile, all while
// the CTA computes the current tile; each is used one tile later, so their
// latency is hidden and no register holds them through the tile.  As in step_kernel_tma there is one barrier between
// two tiles (the copy's arrival), and the previous tile's cells leave by a
// bulk-tensor store issued after it.  Each run of consecutive tiles of one
// problem is reported by every warp on its own (warp_report: atomic maxima
// and counts on the problem's clock, no barrier); the last CTA to leave
// performs the dt shift of every problem of the launch (slots [slot0,
// slot0 + nslots)) and rewinds the counter (counter[0] the claims,
// counter[1] the CTAs that left), so launches follow one another with no
// reset between them.  Copies wait at most `wait_polls` polls (the batch's
// shortest configured wait), then report AST_ST_TIMEOUT to the problem and
// wait with the long limit.
template <int FLUX, bool RECON, bool MIXED>
__global__ void __launch_bounds__(kThreads, 4)
    batch_kernel_tma(const StepParams* __restrict__ Ps, const CUtensorMap* __restrict__ tin,
                     const CUtensorMap* __restrict__ tout, const BatchTile* __restrict__ work, int total, int slot0,
                     int nslots, unsigned int* counter, int wait_polls)
{
    using R = float;
    constexpr int TZ = kTmaTZ, TR = kTmaTR;
    using S = TileSmem<R, MIXED ? 2 : FLUX, TZ, TR, 2>;
    constexpr uint32_t kBoxBytes = 4u * S::HR * S::HZP * sizeof(R);
    constexpr uint32_t kParBytes = sizeof(StepParams);
    static_assert(kParBytes % 16 == 0, "StepParams is copied in 16-byte units");
    S& sm = tile_smem<S>();
    __shared__ __align__(16) StepParams sP[2];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int s_tile[2];
    __shared__ int4 s_work[2];     // {slot | FLUX << 24, n0, m0, 0} of the buffer's tile
    __shared__ int4 s_pend;
    __shared__ StepConsts sK[2];
    __shared__ int s_last;
    // copy thread only: the entry of the next tile to be issued, and per
    // buffer the dt and step of its tile's problem (asynchronous copies)
    __shared__ __align__(16) BatchTile s_next;
    __shared__ double s_tdo[2];
    __shared__ long long s_step[2];
    const int tid = threadIdx.x;
    const bool copier = tid == kCopyThread;
    // the box and the parameters of entry w into buffer bb; its dt and step
    auto issue = [&](int bb, const BatchTile& w) {
        const int jn = w.sf & 0xffffff;
        s_work[bb] = make_int4(w.sf, w.n0, w.m0, 0);
        tma::mbar_expect(&bar[bb], kBoxBytes + kParBytes);
        tma::load_3d(&tin[jn], &sm.qb[bb][0][0][0], &bar[bb], w.n0 - 4, w.m0 - 2, 0);
        tma::load_bulk(&sP[bb], Ps + jn, kParBytes, &bar[bb]);
        tma::async_copy8(&s_tdo[bb], &w.clock->T_do);
        tma::async_copy8(&s_step[bb], &w.clock->step);
    };
    // the entry of work-list tile t into s_next
    auto fetch = [&](int t) {
        tma::async_copy16(&s_next, &work[t]);
        tma::async_copy16(reinterpret_cast<char*>(&s_next) + 16, reinterpret_cast<const char*>(&work[t]) + 16);
    };
    if (copier) {
        tma::mbar_init(&bar[0], 1);
        tma::mbar_init(&bar[1], 1);
        tma::fence_async_shared();
        sm.qn = 0u;
        s_pend = make_int4(-1, 0, 0, 0);
        const int t0 = (int)atomicAdd(counter, 1u);
        s_tile[0] = t0;
        int t1 = total;
        if (t0 < total) {
            const BatchTile w0 = work[t0];
            issue(0, w0);
            t1 = (int)atomicAdd(counter, 1u);
            if (t1 < total) fetch(t1);
        }
        tma::async_commit();
        s_tile[1] = t1;
    }
    __syncthreads();
    phase_mark(kPhaseStart);
    TileAcc<R> acc;
    acc.clear();
    int hb = -1;   // buffer of the last tile computed while its run is not reported yet
    for (int k = 0;; k++) {
        const int b = k & 1;
        if (s_tile[b] >= total) break;
        const int4 w = s_work[b];
        const int j = w.x & 0xffffff, n0 = w.y, m0 = w.z;
        // the one barrier between two tiles: every thread has finished the
        // previous tile (its update, its reads of this buffer's slots) and
        // fenced its shared-memory writes for the bulk copies
        bool arrived = tma::mbar_wait(&bar[b], (uint32_t)((k >> 1) & 1), wait_polls);
        if (__syncthreads_or(!arrived)) {
            // reported (from global memory: the parameters come with the
            // copy), then waited for with the long limit and computed; the
            // next tile's copy is not issued yet, so a copy that does not
            // arrive even then ends this CTA's tiles with none in flight
            if (copier) atomicOr(&Ps[j].clock->status, AST_ST_TIMEOUT);
            arrived = tma::mbar_wait(&bar[b], (uint32_t)((k >> 1) & 1));
            if (__syncthreads_or(!arrived)) break;
        }
        phase_mark(0);
        const StepParams& P = sP[b];
        if (n0 - 2 < 0 || n0 + TZ + 2 > P.N || m0 - 2 < 0 || m0 + TR + 2 > P.M || P.fixed_region) {
            patch_tile<R, TZ, TR>(P, sm, b, n0, m0);
            __syncthreads();
        }
        phase_mark(1);
        int claim = total;
        if (copier) {
            // the asynchronous copies of the previous tile: this tile's dt
            // and step, the next tile's entry
            tma::async_wait_all();
            // the previous tile's cells (sm.out is not written again before
            // the store has read it: see tile_body)
            const int4 pend = s_pend;
            if (pend.x >= 0) {
                tma::store_3d(&tout[pend.x], &sm.out[0][0][0], pend.y, pend.z, 0);
                tma::store_commit();
            }
            s_pend = make_int4(j, n0, m0, 0);
            // the next tile's box, parameters, dt and step into the other
            // buffer (last read by the previous tile), and the claim of the
            // tile after it (its slot written after this tile)
            if (s_tile[b ^ 1] < total) {
                issue(b ^ 1, s_next);
                claim = (int)atomicAdd(counter, 1u);
            }
            // this tile's step constants (read after the face pass's barrier)
            step_consts_of(P, s_tdo[b], (int)s_step[b], sK[b]);
        }
        if constexpr (MIXED) {
            switch (w.x >> 24) {
            case 0: tile_body<R, 0, RECON, kSoA, TZ, TR, true, true, true>(P, sm, b, P.gf, n0, m0, sK[b], acc); break;
            case 1: tile_body<R, 1, RECON, kSoA, TZ, TR, true, true, true>(P, sm, b, P.gf, n0, m0, sK[b], acc); break;
            case 3: tile_body<R, 3, RECON, kSoA, TZ, TR, true, true, true>(P, sm, b, P.gf, n0, m0, sK[b], acc); break;
            default: tile_body<R, 2, RECON, kSoA, TZ, TR, true, true, true>(P, sm, b, P.gf, n0, m0, sK[b], acc); break;
            }
        } else {
            tile_body<R, FLUX, RECON, kSoA, TZ, TR, true, true, true>(P, sm, b, P.gf, n0, m0, sK[b], acc);
        }
        // this thread's shared-memory writes before the bulk copies that
        // read or overwrite them (ordered by the next barrier)
        tma::fence_async_shared();
        if (copier) {
            // read at the top of the iteration after next, after barriers
            s_tile[b] = claim;
            if (claim < total) fetch(claim);
            tma::async_commit();
        }
        hb = b;
        // the run ends when the next tile is another problem's: s_tile[b ^ 1]
        // was written before the previous barrier, s_work[b ^ 1] before this
        // tile's face-pass barrier, so every thread takes the same branch
        if (s_tile[b ^ 1] >= total || (s_work[b ^ 1].x & 0xffffff) != j) {
            warp_report<R>(P, acc);
            acc.clear();
            hb = -1;
            phase_mark(5);
        }
    }
    // a run left unreported when a copy never arrived
    if (hb >= 0) warp_report<R>(sP[hb], acc);
    phase_mark(5);
    __syncthreads();
    if (copier) {
        // (asynchronous copies still in flight when a copy never arrived)
        tma::async_wait_all();
        const int4 pend = s_pend;
        if (pend.x >= 0) {
            tma::store_3d(&tout[pend.x], &sm.out[0][0][0], pend.y, pend.z, 0);
            tma::store_commit();
        }
        tma::store_wait_all();
        // every claim and report of this CTA is made: the last CTA to leave
        // shifts the problems' clocks and rewinds the counter
        __threadfence();
        s_last = (atomicAdd(counter + 1, 1u) == gridDim.x - 1) ? 1 : 0;
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int p = slot0 + tid; p < slot0 + nslots; p += kThreads) clock_shift(Ps[p]);
        if (tid == 0) {
            counter[0] = 0u;
            counter[1] = 0u;
        }
    }
#ifdef AST_PHASE_CLOCKS
    phase_mark(kPhaseFlush, Ps[slot0].clock);
#endif
}

// Characteristic inflow at z_lo after a step (add2_bound, kernel.cu:1895-
// 1925): one thread per row m; from the old state of cell (0, m) (P.in)
// and the new state of cell (1, m) (P.out), cell (0, m) of P.out becomes
// rho = pp/(gamma-1)/T0, p = p_in, (v_z, v_r) = (v_in, 0), with
// T0 = p_in/(gamma-1) and pp = p'(1) - rho(0) c(0) (v_z'(1) - v_in).
// separately rounded multiply / subtract / divide (no contraction into an
// FMA), for the few operations per row of the inflow rule
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

template <typename R, int LAYOUT>
__global__ void inflow_kernel(StepParams P, double p_in, double v_in)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= P.M) return;
    const Gas<R>& g = gas_of<R>(P);
    R r0, p0, p1, u1;
    if (LAYOUT == kSoA) {
        const R* q = (const R*)P.in;
        const R* o = (const R*)P.out;
        const long long k = (long long)m * P.ld;
        r0 = q[k]; p0 = q[k + P.plane];
        p1 = o[k + 1 + P.plane]; u1 = o[k + 1 + 2 * P.plane];
    } else {
        const long long k = (long long)m * P.N;
        const double2 s0 = ((const double2*)P.in)[k];
        r0 = (R)s0.x; p0 = (R)s0.y;
        p1 = (R)((const double2*)P.out)[k + 1].y;
        u1 = (R)((const double2*)P.out_u)[k + 1].x;
    }
    const R cc = sqrt(div_rn(mul_rn(g.ga, p0), r0));
    const R T0 = div_rn(div_rn((R)p_in, g.g1), R(1));
    const R pp = sub_rn(p1, mul_rn(mul_rn(r0, cc), sub_rn(u1, (R)v_in)));
    const R rho = div_rn(div_rn(pp, g.g1), T0);
    if (LAYOUT == kSoA) {
        R* o = (R*)P.out;
        const long long k = (long long)m * P.ld;
        o[k] = rho; o[k + P.plane] = (R)p_in; o[k + 2 * P.plane] = (R)v_in; o[k + 3 * P.plane] = R(0);
    } else {
        const long long k = (long long)m * P.N;
        ((double2*)P.out)[k] = make_double2((double)rho, p_in);
        ((double2*)P.out_u)[k] = make_double2(v_in, 0.0);
    }
}

}  // namespace ast
