// api.cu - the C ABI of include/asteriy_gb300.h on top of the step kernel.
//
// The solver object replaces the reference's main(): allocation
// (kernel.cu:3283-3298), host->device copies (kernel.cu:3444-3455), the
// ping-pong time loop with its funk_time launches and synchronisations
// (kernel.cu:3868-3947) and the final device->host copies
// (kernel.cu:4075-4080).  Steps are queued on one stream; the dt shift runs
// on the device inside the step kernel, so nsteps steps cost nsteps launches
// and no host synchronisation.  Repeated step counts are replayed from a
// captured CUDA graph.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "../../include/asteriy_gb300.h"
#include "convert.cuh"
#include "launch.cuh"

using namespace ast;

namespace {

thread_local std::string g_last_error;

#define AST_CUDA(call)                                      \
    do {                                                    \
        cudaError_t e_ = (call);                            \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call); \
    } while (0)

int fail(int code, const char* msg)
{
    g_last_error = msg;
    return code;
}

// density of the state planes q at cells k = m*N + n
template <typename R>
__global__ void probe_kernel(const R* __restrict__ q, long long ld, int N, const int64_t* __restrict__ cells, int n,
                             double* __restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long k = cells[i];
    const long long m = k / N, c = k - m * N;
    out[i] = (double)q[m * ld + c];
}

__global__ void funk_time_kernel(double* T, double* T_do, double* TT, int* i)
{
    *T_do = *T;
    *TT = *TT + *T_do;
    *T = 10000000;
    *i = *i + 1;
}

}  // namespace

int ast::cuda_fail(cudaError_t e, const char* what)
{
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return AST_ERR_CUDA;
}

int ast::set_error(int code, const char* msg) { return fail(code, msg); }

// the four FP32 state planes of one time level as a 3-D tensor (x = z
// cells, y = rows, z = planes) with a TMA box of `bx` x `by` x 4
int ast::encode_planes(CUtensorMap* map, void* base, const ast_config& c, long long ld, long long plane, unsigned bx,
                       unsigned by)
{
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return fail(AST_ERR_UNSUPPORTED, "cuTensorMapEncodeTiled not available");
        encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    // FP32 or FP64 state planes
    const bool f64 = c.precision == AST_PREC_FP64;
    const size_t es = f64 ? sizeof(double) : sizeof(float);
    const cuuint64_t dim[3] = {(cuuint64_t)c.N, (cuuint64_t)c.M, 4};
    const cuuint64_t stride[2] = {(cuuint64_t)ld * es, (cuuint64_t)plane * es};
    const cuuint32_t box[3] = {bx, by, 4};
    const cuuint32_t estride[3] = {1, 1, 1};
    CUresult r = encode(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dim,
                        stride, box, estride,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? AST_OK : fail(AST_ERR_CUDA, "cuTensorMapEncodeTiled failed");
}

// ==================================================================== solver
struct ast_solver {
    ast_config cfg;
    StepParams P;
    cudaStream_t stream = nullptr;
    size_t elem = 8;                 // bytes per state value
    long long ld = 0, plane = 0;
    void* buf[2] = {nullptr, nullptr};
    int cur = 0;
    DevClock* clock = nullptr;
    double* stage_s = nullptr;       // device AoS staging for set/get
    double* stage_u = nullptr;
    cudaGraphExec_t graph = nullptr; // captured block of graph_steps steps
    int graph_steps = 0;
    int graph_cur = -1;              // buffer index the graph starts from
    float* mlp = nullptr;            // learned start value parameters (device)
    float* rec = nullptr;            // face recorder buffer (device)
    unsigned long long* rec_n = nullptr;
    long long rec_cap = 0;
    int64_t* probe_buf = nullptr;    // watch cells (device): n indices, then n doubles
    int probe_cap = 0;
    bool tma = false;                // FP32 persistent kernel
    int tma_grid = 0;                // its CTAs
    bool sweep = false;              // FP32 strip kernel
    int sweep_grid = 0;              // its CTAs (at most)
    CUtensorMap tin[2], tout[2];     // tile-box load and store maps of buf[0], buf[1]
    void* nsrc = nullptr;            // neutral-coupling source planes (nn2.x, nn2.y), or null
    double* q[2] = {nullptr, nullptr};   // the passive scalar, per time level (N*M, row-major), or null
    bool has_q = false;
    cudaStream_t pipe[2] = {nullptr, nullptr};   // ast_step_host: copies in, copies out
    cudaEvent_t pev[3 * 16 + 2] = {};            // its band events (created on first use)
};

extern "C" {

int ast_abi_version(void) { return AST_ABI_VERSION; }

const char* ast_last_error(void) { return g_last_error.c_str(); }

const char* ast_strerror(int code)
{
    switch (code) {
    case AST_OK: return "ok";
    case AST_ERR_INVALID: return "invalid argument or configuration";
    case AST_ERR_CUDA: return "CUDA runtime error";
    case AST_ERR_NOMEM: return "out of memory";
    case AST_ERR_IO: return "file I/O error";
    case AST_ERR_UNSUPPORTED: return "unsupported request";
    case AST_ERR_NUMERIC: return "non-finite values in the state";
    default: return "unknown error";
    }
}

size_t ast_sizeof_config(void) { return sizeof(ast_config); }
size_t ast_sizeof_stats(void) { return sizeof(ast_stats); }

int ast_create(const ast_config* cfg, ast_solver** out)
{
    if (!cfg || !out) return fail(AST_ERR_INVALID, "null argument");
    *out = nullptr;
    int rc = ast_config_check(cfg);
    if (rc != AST_OK) return rc;
    ast_solver* S = new (std::nothrow) ast_solver();
    if (!S) return fail(AST_ERR_NOMEM, "host allocation");
    S->cfg = *cfg;
    S->elem = (cfg->precision == AST_PREC_FP32) ? 4 : 8;
    // rows padded to 128 bytes: aligned, coalesced row starts
    const long long align = 128 / (long long)S->elem;
    S->ld = ((long long)cfg->N + align - 1) / align * align;
    S->plane = S->ld * cfg->M;
    const size_t bytes = (size_t)S->plane * 4 * S->elem;
    const size_t K = (size_t)cfg->N * cfg->M;
    cudaError_t e;
    if ((e = cudaMalloc(&S->buf[0], bytes)) != cudaSuccess || (e = cudaMalloc(&S->buf[1], bytes)) != cudaSuccess ||
        (e = cudaMalloc(&S->clock, sizeof(DevClock))) != cudaSuccess ||
        (e = cudaMalloc(&S->stage_s, K * 2 * sizeof(double))) != cudaSuccess ||
        (e = cudaMalloc(&S->stage_u, K * 2 * sizeof(double))) != cudaSuccess) {
        ast_destroy(S);
        g_last_error = std::string("cudaMalloc: ") + cudaGetErrorString(e);
        return AST_ERR_NOMEM;
    }
    cudaMemset(S->buf[0], 0, bytes);
    cudaMemset(S->buf[1], 0, bytes);
    fill_step_params(S->P, *cfg);
    S->P.ld = S->ld;
    S->P.plane = S->plane;
    S->P.clock = S->clock;
    DevClock c0;
    std::memset(&c0, 0, sizeof c0);
    c0.T_do = cfg->dt_first;
    if ((e = cudaMemcpy(S->clock, &c0, sizeof c0, cudaMemcpyHostToDevice)) != cudaSuccess) {
        ast_destroy(S);
        return cuda_fail(e, "cudaMemcpy clock");
    }
    rc = (S->elem == 8) ? launch_step_r<double, kSoA>(S->P, cfg->flux, cfg->recon, nullptr, false)
                        : launch_step_r<float, kSoA>(S->P, cfg->flux, cfg->recon, nullptr, false);
    // FP32: the strip kernel (persistent = 2) or the persistent tile kernel (1)
    const bool want_sweep = S->elem == 4 && cfg->persistent == 2;
    if (rc == AST_OK && want_sweep) {
        int per_sm = 0, dev = 0, sms = 0;
        rc = launch_step_sweep(S->P, cfg->flux, cfg->recon, 0, nullptr, false, &per_sm);
        if (rc == AST_OK && (e = cudaGetDevice(&dev)) != cudaSuccess) rc = cuda_fail(e, "cudaGetDevice");
        if (rc == AST_OK && (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            rc = cuda_fail(e, "cudaDeviceGetAttribute");
        if (rc == AST_OK) {
            const int strips = sweep_strips(cfg->N, cfg->M, 0, 0);
            S->sweep_grid = std::min((strips + kThreads / 32 - 1) / (kThreads / 32), std::max(per_sm, 1) * sms);
            S->sweep = true;
        }
    }
    // FP64: the persistent kernel for the HLL family on grids of at least
    // two 32x16 tiles per SM (smaller grids step with one CTA per tile of
    // 16x16).  The exact solver keeps one CTA per tile: for it the
    // persistent kernel measured 8% slower (11.32 against 10.44 ms per step
    // at step 1000 of the 4096x2048 blast; HLL 4.79 against 5.20 ms), and
    // 10% slower again with today's face pass (11.02 against 10.03 ms).
    const long long tiles32 = (long long)((cfg->N + kTZ - 1) / kTZ) * ((cfg->M + kTR - 1) / kTR);
    const bool tma64 = S->elem == 8 && cfg->flux != AST_FLUX_GODUNOV && tiles32 >= 2LL * sm_count();
    if (rc == AST_OK && (S->elem == 4 || tma64) && cfg->persistent && !want_sweep) {
        // box loads of tile + halo (TZ+8 x TR+4), stores of the tile (TZ x TR)
        for (int b = 0; b < 2 && rc == AST_OK; b++) {
            rc = encode_planes(&S->tin[b], S->buf[b], *cfg, S->ld, S->plane, kTZ + 8, kTR + 4);
            if (rc == AST_OK) rc = encode_planes(&S->tout[b], S->buf[b], *cfg, S->ld, S->plane, kTZ, kTR);
        }
        int per_sm = 0, dev = 0, sms = 0;
        if (rc == AST_OK)
            rc = launch_step_tma_e(S->elem, S->P, S->tin[0], S->tout[1], cfg->flux, cfg->recon, 0, nullptr, false,
                                   &per_sm);
        if (rc == AST_OK && (e = cudaGetDevice(&dev)) != cudaSuccess) rc = cuda_fail(e, "cudaGetDevice");
        if (rc == AST_OK && (e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
            rc = cuda_fail(e, "cudaDeviceGetAttribute");
        if (rc == AST_OK) {
            const long long tiles = (long long)((cfg->N + kTZ - 1) / kTZ) * ((cfg->M + kTR - 1) / kTR);
            S->tma_grid = (int)std::min<long long>(tiles, (long long)std::max(per_sm, 1) * sms);
            S->tma = true;
        }
    }
    if (rc != AST_OK) {
        ast_destroy(S);
        return rc;
    }
    *out = S;
    return AST_OK;
}

int ast_destroy(ast_solver* S)
{
    if (!S) return AST_OK;
    if (S->graph) cudaGraphExecDestroy(S->graph);
    for (cudaEvent_t& ev : S->pev)
        if (ev) cudaEventDestroy(ev);
    for (cudaStream_t& st : S->pipe)
        if (st) cudaStreamDestroy(st);
    cudaFree(S->buf[0]);
    cudaFree(S->buf[1]);
    cudaFree(S->clock);
    cudaFree(S->stage_s);
    cudaFree(S->stage_u);
    cudaFree(S->mlp);
    cudaFree(S->rec);
    cudaFree(S->rec_n);
    cudaFree(S->probe_buf);
    cudaFree(S->nsrc);
    cudaFree(S->q[0]);
    cudaFree(S->q[1]);
    delete S;
    return AST_OK;
}

int ast_set_stream(ast_solver* S, void* stream)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    S->stream = (cudaStream_t)stream;
    if (S->graph) {
        cudaGraphExecDestroy(S->graph);
        S->graph = nullptr;
    }
    return AST_OK;
}

// The device address of the host range [p, p + bytes) when the GPU can
// read and write it in place: page-locked host memory (over NVLink-C2C on
// GB300), the whole range inside one allocation.  Otherwise nullptr, and
// the caller copies through its device staging buffers.
static void* host_range_on_device(const void* p, size_t bytes)
{
    using GetAttr = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
    static GetAttr get = nullptr;
    static bool looked = false;
    if (!looked) {
        looked = true;
        cudaDriverEntryPointQueryResult q;
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 4000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get = reinterpret_cast<GetAttr>(fn);
        cudaGetLastError();
    }
    if (!get) return nullptr;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr) return nullptr;
    CUdeviceptr start = 0;
    size_t size = 0;
    const CUdeviceptr d = (CUdeviceptr)a.devicePointer;
    if (get(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, d) != CUDA_SUCCESS) return nullptr;
    if (get(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, d) != CUDA_SUCCESS) return nullptr;
    if (d < start || d + bytes > start + size) return nullptr;
    return a.devicePointer;
}

static int convert_in(ast_solver* S, const double* s, const double* u)
{
    const long long K = (long long)S->cfg.N * S->cfg.M;
    const int nb = (int)((K + 255) / 256);
    void* dst = S->buf[S->cur];
    if (S->elem == 8)
        aos_to_soa<double><<<nb, 256, 0, S->stream>>>((const double2*)s, (const double2*)u, (double*)dst, S->cfg.N,
                                                      S->cfg.M, S->ld, S->plane);
    else
        aos_to_soa<float><<<nb, 256, 0, S->stream>>>((const double2*)s, (const double2*)u, (float*)dst, S->cfg.N,
                                                     S->cfg.M, S->ld, S->plane);
    AST_CUDA(cudaGetLastError());
    return AST_OK;
}

int ast_set_state(ast_solver* S, const double* s, const double* u, int on_device)
{
    if (!S || !s || !u) return fail(AST_ERR_INVALID, "null argument");
    const size_t bytes = (size_t)S->cfg.N * S->cfg.M * 2 * sizeof(double);
    if (on_device) return convert_in(S, s, u);
    // page-locked host arrays: the conversion kernel reads them in place
    const void* ds = host_range_on_device(s, bytes);
    const void* du = ds ? host_range_on_device(u, bytes) : nullptr;
    if (ds && du) {
        int rc = convert_in(S, (const double*)ds, (const double*)du);
        if (rc != AST_OK) return rc;
        AST_CUDA(cudaStreamSynchronize(S->stream));
        return AST_OK;
    }
    AST_CUDA(cudaMemcpyAsync(S->stage_s, s, bytes, cudaMemcpyHostToDevice, S->stream));
    AST_CUDA(cudaMemcpyAsync(S->stage_u, u, bytes, cudaMemcpyHostToDevice, S->stream));
    int rc = convert_in(S, S->stage_s, S->stage_u);
    if (rc != AST_OK) return rc;
    AST_CUDA(cudaStreamSynchronize(S->stream));
    return AST_OK;
}

int ast_get_state(ast_solver* S, double* s, double* u, int on_device)
{
    if (!S || !s || !u) return fail(AST_ERR_INVALID, "null argument");
    const long long K = (long long)S->cfg.N * S->cfg.M;
    const int nb = (int)((K + 255) / 256);
    const size_t bytes = (size_t)K * 2 * sizeof(double);
    // page-locked host arrays: the conversion kernel writes them in place
    double* hs = on_device ? nullptr : (double*)host_range_on_device(s, bytes);
    double* hu = hs ? (double*)host_range_on_device(u, bytes) : nullptr;
    const bool direct = on_device || (hs && hu);
    double* ds = on_device ? s : (direct ? hs : S->stage_s);
    double* du = on_device ? u : (direct ? hu : S->stage_u);
    const void* src = S->buf[S->cur];
    if (S->elem == 8)
        soa_to_aos<double><<<nb, 256, 0, S->stream>>>((const double*)src, (double2*)ds, (double2*)du, S->cfg.N,
                                                      S->cfg.M, S->ld, S->plane);
    else
        soa_to_aos<float><<<nb, 256, 0, S->stream>>>((const float*)src, (double2*)ds, (double2*)du, S->cfg.N,
                                                     S->cfg.M, S->ld, S->plane);
    AST_CUDA(cudaGetLastError());
    if (!on_device) {
        if (!direct) {
            AST_CUDA(cudaMemcpyAsync(s, ds, bytes, cudaMemcpyDeviceToHost, S->stream));
            AST_CUDA(cudaMemcpyAsync(u, du, bytes, cudaMemcpyDeviceToHost, S->stream));
        }
        AST_CUDA(cudaStreamSynchronize(S->stream));
    }
    return AST_OK;
}

int ast_set_clock(ast_solver* S, double T_do, double TT, int64_t step)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    DevClock c;
    AST_CUDA(cudaMemcpyAsync(&c, S->clock, sizeof c, cudaMemcpyDeviceToHost, S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    c.T_do = T_do;
    c.TT = TT;
    c.step = step;
    c.smax_z = c.smax_r = 0;
    c.done = 0;
    AST_CUDA(cudaMemcpyAsync(S->clock, &c, sizeof c, cudaMemcpyHostToDevice, S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    return AST_OK;
}

int ast_get_clock(ast_solver* S, double* T_do, double* TT, int64_t* step)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    DevClock c;
    AST_CUDA(cudaMemcpyAsync(&c, S->clock, sizeof c, cudaMemcpyDeviceToHost, S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    if (T_do) *T_do = c.T_do;
    if (TT) *TT = c.TT;
    if (step) *step = c.step;
    return AST_OK;
}

// The FP32 form's neutral-coupling source, after the step (P.in: the state
// the step read, P.out: the state it wrote; SoA planes): the momentum
// T_do * (rho * coef) * (nn2.x, nn2.y) of add_MK (kernel.cu:2495-2496),
// rho the old density, T_do the step's dt, added to the new momentum at
// fixed total energy (add_MK's energy term is zero), in FP64:
// v += S / rho', p -= (gamma - 1) rho' (|v + S/rho'|^2 - |v|^2) / 2, then
// the pressure floor.  Cells of the fixed region are left as they are.
// In the kernel the source term would cost the FP32 update registers and
// time (2% at 4096x2048) on every step, used or not.
static __global__ void neutral_kernel(StepParams P)
{
    const long long K = (long long)P.N * P.M;
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < K; k += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(k / P.N), n = (int)(k - (long long)m * P.N);
        if (P.fixed_region && n >= P.fixed_nlo && n <= P.fixed_nhi && m <= P.fixed_mhi &&
            cell_fixed(P, P.x_min + n * P.dx, P.y_min + m * P.dy))
            continue;
        const long long j = (long long)m * P.ld + n;
        const float* q = (const float*)P.in;
        float* o = (float*)P.out;
        const float* src = (const float*)P.nsrc;
        const double T = P.clock->T_prev;
        const double rho2 = o[j], vz = o[j + 2 * P.plane], vr = o[j + 3 * P.plane];
        const double w = T * ((double)q[j] * P.nsrc_coef) / rho2;
        const double vz2 = vz + w * (double)src[j], vr2 = vr + w * (double)src[j + P.plane];
        double p2 = (double)o[j + P.plane] - P.gd.g1 * 0.5 * rho2 * ((vz2 * vz2 + vr2 * vr2) - (vz * vz + vr * vr));
        if (p2 <= 0.0) p2 = P.p_floor;
        o[j + P.plane] = (float)p2;
        o[j + 2 * P.plane] = (float)vz2;
        o[j + 3 * P.plane] = (float)vr2;
    }
}

// CTAs of the strip kernel for tile rows [t0, t1): one per 8 strips, at
// most the solver's grid
static int band_sweep_grid(const ast_solver* S, int t0, int t1)
{
    const int strips = sweep_strips(S->cfg.N, S->cfg.M, t0, t1);
    return std::min((strips + kThreads / 32 - 1) / (kThreads / 32), S->sweep_grid);
}

static int enqueue_one(ast_solver* S)
{
    StepParams P = S->P;
    P.in = S->buf[S->cur];
    P.out = S->buf[S->cur ^ 1];
    int rc;
    // the passive scalar first: it reads the old state and this step's dt,
    // which the gas step's epilogue replaces
    if (S->has_q) {
        rc = launch_scalar(P, S->q[S->cur], S->q[S->cur ^ 1], S->cfg.flux, S->cfg.recon, S->cfg.scalar_in, S->stream);
        if (rc != AST_OK) return rc;
    }
    if (S->sweep)
        rc = launch_step_sweep(P, S->cfg.flux, S->cfg.recon, S->sweep_grid, S->stream, true, nullptr);
    else if (S->tma)
        rc = launch_step_tma_e(S->elem, P, S->tin[S->cur], S->tout[S->cur ^ 1], S->cfg.flux, S->cfg.recon,
                               S->tma_grid, S->stream, true, nullptr);
    else
        rc = (S->elem == 8) ? launch_step_r<double, kSoA>(P, S->cfg.flux, S->cfg.recon, S->stream, true)
                            : launch_step_r<float, kSoA>(P, S->cfg.flux, S->cfg.recon, S->stream, true);
    if (rc == AST_OK && S->elem == 4 && P.nsrc) {
        // the FP32 form's neutral-coupling source, after the step
        const long long K = (long long)S->cfg.N * S->cfg.M;
        const int nb = (int)std::min<long long>((K + 255) / 256, 16LL * sm_count());
        neutral_kernel<<<nb, 256, 0, S->stream>>>(P);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "neutral source kernel launch");
    }
    if (rc == AST_OK && S->cfg.inflow_p > 0.0) {
        const int nb = (S->cfg.M + 127) / 128;
        if (S->elem == 8)
            inflow_kernel<double, kSoA><<<nb, 128, 0, S->stream>>>(P, S->cfg.inflow_p, S->cfg.inflow_v);
        else
            inflow_kernel<float, kSoA><<<nb, 128, 0, S->stream>>>(P, S->cfg.inflow_p, S->cfg.inflow_v);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda_fail(e, "inflow kernel launch");
    }
    if (rc == AST_OK) S->cur ^= 1;
    return rc;
}

// Captures `count` consecutive steps starting from buffer `cur` into a graph.
static int capture_block(ast_solver* S, int count)
{
    if (S->graph) {
        cudaGraphExecDestroy(S->graph);
        S->graph = nullptr;
    }
    cudaStream_t cs;
    AST_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaStream_t saved = S->stream;
    const int cur0 = S->cur;
    S->stream = cs;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    int rc = AST_OK;
    if (e == cudaSuccess) {
        for (int i = 0; i < count && rc == AST_OK; i++) rc = enqueue_one(S);
        e = cudaStreamEndCapture(cs, &graph);
    }
    S->stream = saved;
    S->cur = cur0;
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return cuda_fail(e, "graph capture");
    if (rc != AST_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    e = cudaGraphInstantiate(&S->graph, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    S->graph_steps = count;
    S->graph_cur = cur0;
    return AST_OK;
}

int ast_step(ast_solver* S, int nsteps)
{
    if (!S || nsteps < 0) return fail(AST_ERR_INVALID, "bad argument");
    if (S->cfg.flux == AST_FLUX_GODUNOV && S->cfg.guess == AST_GUESS_MLP && S->P.riemann_newton && !S->mlp)
        return fail(AST_ERR_INVALID, "guess == MLP needs ast_set_mlp first");
    // a captured block of an even number of steps returns to the same
    // buffer, so it can be replayed back to back
    const int block = 16;
    while (nsteps >= block) {
        if (!S->graph || S->graph_steps != block || S->graph_cur != S->cur) {
            int rc = capture_block(S, block);
            if (rc != AST_OK) return rc;
        }
        AST_CUDA(cudaGraphLaunch(S->graph, S->stream));
        nsteps -= block;
    }
    for (int i = 0; i < nsteps; i++) {
        int rc = enqueue_one(S);
        if (rc != AST_OK) return rc;
    }
    return AST_OK;
}

// ast_step_host / ast_step_host_n: steps from host arrays to host arrays,
// pipelined over bands of tile rows.  Two copy streams carry nothing but
// copies, so the host link's two directions stay busy: `in` copies band b's
// s, u into the device staging arrays, `out` copies band b of the new state
// back.  The kernels run in order on the solver's stream: band b + 1
// converted into the state buffer (it holds band b's lower halo rows), band
// b stepped, band b converted into staging for `out`.  Over several steps
// band b of step k + 1 goes in as soon as band b of step k is out (its
// input is that output, and it reuses those staging rows), so the copies
// of consecutive steps overlap too.
static constexpr int kHostBands = 16, kChainBands = 4;

static bool ranges_overlap(const void* a, const void* b, size_t bytes)
{
    const char *x = (const char*)a, *y = (const char*)b;
    return x < y + bytes && y < x + bytes;
}

// nsteps steps, step k reading (s_a, u_a) for even k and (s_b, u_b) for odd
// k and writing the other pair
static int host_steps(ast_solver* S, int nsteps, double* s_a, double* u_a, double* s_b, double* u_b)
{
    if (!S || !s_a || !u_a || !s_b || !u_b || nsteps < 0) return fail(AST_ERR_INVALID, "bad argument");
    if (S->cfg.flux == AST_FLUX_GODUNOV && S->cfg.guess == AST_GUESS_MLP && S->P.riemann_newton && !S->mlp)
        return fail(AST_ERR_INVALID, "guess == MLP needs ast_set_mlp first");
    if (S->has_q) return fail(AST_ERR_UNSUPPORTED, "the host-array steps do not carry the passive scalar");
    const int N = S->cfg.N, M = S->cfg.M;
    const size_t bytes = (size_t)N * M * 2 * sizeof(double);
    // a pair's arrays lie apart; an array of one pair is an array of the
    // other (in place) or lies apart from both: band b's results are written
    // after the inputs of all bands up to b + 1 were read, but before those
    // of later bands
    if (ranges_overlap(s_a, u_a, bytes) || ranges_overlap(s_b, u_b, bytes))
        return fail(AST_ERR_INVALID, "overlapping host arrays");
    for (const double* o : {(const double*)s_b, (const double*)u_b})
        for (const double* i : {(const double*)s_a, (const double*)u_a})
            if (o != i && ranges_overlap(o, i, bytes)) return fail(AST_ERR_INVALID, "overlapping host arrays");
    if (nsteps == 0) return AST_OK;
    const bool pinned = host_range_on_device(s_a, bytes) && host_range_on_device(u_a, bytes) &&
                        host_range_on_device(s_b, bytes) && host_range_on_device(u_b, bytes);
    if (!pinned || S->cfg.inflow_p > 0.0 || (S->elem == 4 && S->P.nsrc)) {
        // pageable arrays (the copies would not overlap), or a pass over
        // every row after the step (the inflow rule, the FP32 form's
        // neutral-coupling source): the three calls in turn
        for (int k = 0; k < nsteps; k++) {
            const bool odd = k & 1;
            int rc = ast_set_state(S, odd ? s_b : s_a, odd ? u_b : u_a, 0);
            if (rc == AST_OK) rc = ast_step(S, 1);
            if (rc == AST_OK) rc = ast_get_state(S, odd ? s_a : s_b, odd ? u_a : u_b, 0);
            if (rc != AST_OK) return rc;
        }
        return AST_OK;
    }
    if (!S->pipe[0]) {
        for (cudaStream_t& st : S->pipe) AST_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        for (cudaEvent_t& ev : S->pev) AST_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    }
    // bands: one step waits for its first two bands to come in and for its
    // last band to go out, so a single step wants small bands (16: 2.03 ms
    // per step at 4096x2048, 4: 2.27 ms); a chain of steps keeps both
    // directions busy across steps and wants few, large copies (4 bands:
    // 1.65 ms per step, 16: 1.85 ms)
    const int rows = (M + kTR - 1) / kTR;   // tile rows
    const int bands = std::min(rows, nsteps > 1 ? kChainBands : kHostBands);
    cudaEvent_t* ev_in = S->pev;                      // band b in staging
    cudaEvent_t* ev_out = S->pev + kHostBands;        // band b of the new state in staging
    cudaEvent_t* ev_back = S->pev + 2 * kHostBands;   // band b of the new state in host memory
    cudaEvent_t ev_start = S->pev[3 * kHostBands], ev_done = S->pev[3 * kHostBands + 1];
    cudaStream_t cin = S->pipe[0], cst = S->stream, cout = S->pipe[1];
    struct Band {
        int t0, t1;          // tile rows
        long long k0, k1;    // cells
    };
    Band bd[kHostBands];
    const int tiles_z = (N + kTZ - 1) / kTZ;
    int units = 0;   // CTAs of all bands' persistent launches
    for (int b = 0; b < bands; b++) {
        bd[b].t0 = (int)((long long)b * rows / bands);
        bd[b].t1 = (int)((long long)(b + 1) * rows / bands);
        bd[b].k0 = (long long)bd[b].t0 * kTR * N;
        bd[b].k1 = (long long)std::min(bd[b].t1 * kTR, M) * N;
        units += S->sweep ? band_sweep_grid(S, bd[b].t0, bd[b].t1)
                          : std::min((bd[b].t1 - bd[b].t0) * tiles_z, S->tma_grid);
    }
    AST_CUDA(cudaEventRecord(ev_start, cst));
    AST_CUDA(cudaStreamWaitEvent(cin, ev_start, 0));
    AST_CUDA(cudaStreamWaitEvent(cout, ev_start, 0));
    int rc = AST_OK;
    for (int k = 0; k < nsteps && rc == AST_OK; k++) {
        const bool odd = k & 1;
        const double* s_in = odd ? s_b : s_a;
        const double* u_in = odd ? u_b : u_a;
        double* s_out = odd ? s_a : s_b;
        double* u_out = odd ? u_a : u_b;
        for (int b = 0; b < bands; b++) {
            // step k's input of band b is step k - 1's output of band b,
            // and the staging rows are free once that output has left them
            if (k > 0) AST_CUDA(cudaStreamWaitEvent(cin, ev_back[b], 0));
            const size_t off = (size_t)bd[b].k0 * 2, n = (size_t)(bd[b].k1 - bd[b].k0) * 2 * sizeof(double);
            AST_CUDA(cudaMemcpyAsync(S->stage_s + off, s_in + off, n, cudaMemcpyHostToDevice, cin));
            AST_CUDA(cudaMemcpyAsync(S->stage_u + off, u_in + off, n, cudaMemcpyHostToDevice, cin));
            AST_CUDA(cudaEventRecord(ev_in[b], cin));
        }
        void* src = S->buf[S->cur];
        void* dst = S->buf[S->cur ^ 1];
        auto convert_band_in = [&](int b) -> int {
            AST_CUDA(cudaStreamWaitEvent(cst, ev_in[b], 0));
            const int nb = (int)((bd[b].k1 - bd[b].k0 + 255) / 256);
            if (S->elem == 8)
                aos_to_soa<double><<<nb, 256, 0, cst>>>((const double2*)S->stage_s, (const double2*)S->stage_u,
                                                        (double*)src, N, M, S->ld, S->plane, bd[b].k0, bd[b].k1);
            else
                aos_to_soa<float><<<nb, 256, 0, cst>>>((const double2*)S->stage_s, (const double2*)S->stage_u,
                                                       (float*)src, N, M, S->ld, S->plane, bd[b].k0, bd[b].k1);
            AST_CUDA(cudaGetLastError());
            return AST_OK;
        };
        rc = convert_band_in(0);
        for (int b = 0; b < bands && rc == AST_OK; b++) {
            if (b + 1 < bands) rc = convert_band_in(b + 1);
            if (rc != AST_OK) break;
            StepParams P = S->P;
            P.in = src;
            P.out = dst;
            P.band_lo = bd[b].t0;
            P.band_hi = bd[b].t1;
            if (S->sweep) {
                // each band hands out its strips from a counter set to zero
                P.units = units;
                if (b > 0) AST_CUDA(cudaMemsetAsync(&S->clock->next_tile, 0, sizeof(unsigned int), cst));
                rc = launch_step_sweep(P, S->cfg.flux, S->cfg.recon, band_sweep_grid(S, bd[b].t0, bd[b].t1), cst,
                                       true, nullptr);
            } else if (S->tma) {
                // each band hands out its tiles from a counter set to zero
                P.units = units;
                if (b > 0) AST_CUDA(cudaMemsetAsync(&S->clock->next_tile, 0, sizeof(unsigned int), cst));
                rc = launch_step_tma_e(S->elem, P, S->tin[S->cur], S->tout[S->cur ^ 1], S->cfg.flux, S->cfg.recon,
                                       std::min((bd[b].t1 - bd[b].t0) * tiles_z, S->tma_grid), cst, true, nullptr);
            } else {
                rc = (S->elem == 8) ? launch_step_r<double, kSoA>(P, S->cfg.flux, S->cfg.recon, cst, true)
                                    : launch_step_r<float, kSoA>(P, S->cfg.flux, S->cfg.recon, cst, true);
            }
            if (rc != AST_OK) break;
            const int nb = (int)((bd[b].k1 - bd[b].k0 + 255) / 256);
            if (S->elem == 8)
                soa_to_aos<double><<<nb, 256, 0, cst>>>((const double*)dst, (double2*)S->stage_s,
                                                        (double2*)S->stage_u, N, M, S->ld, S->plane, bd[b].k0,
                                                        bd[b].k1);
            else
                soa_to_aos<float><<<nb, 256, 0, cst>>>((const float*)dst, (double2*)S->stage_s,
                                                       (double2*)S->stage_u, N, M, S->ld, S->plane, bd[b].k0,
                                                       bd[b].k1);
            AST_CUDA(cudaGetLastError());
            AST_CUDA(cudaEventRecord(ev_out[b], cst));
            const size_t off = (size_t)bd[b].k0 * 2, n = (size_t)(bd[b].k1 - bd[b].k0) * 2 * sizeof(double);
            AST_CUDA(cudaStreamWaitEvent(cout, ev_out[b], 0));
            AST_CUDA(cudaMemcpyAsync(s_out + off, S->stage_s + off, n, cudaMemcpyDeviceToHost, cout));
            AST_CUDA(cudaMemcpyAsync(u_out + off, S->stage_u + off, n, cudaMemcpyDeviceToHost, cout));
            AST_CUDA(cudaEventRecord(ev_back[b], cout));
        }
        if (rc == AST_OK) S->cur ^= 1;
    }
    // the copy streams rejoin the solver's stream even after a failed launch
    AST_CUDA(cudaEventRecord(ev_done, cout));
    AST_CUDA(cudaStreamWaitEvent(cst, ev_done, 0));
    AST_CUDA(cudaEventRecord(ev_done, cin));
    AST_CUDA(cudaStreamWaitEvent(cst, ev_done, 0));
    if (rc != AST_OK) {
        cudaStreamSynchronize(cst);
        return rc;
    }
    AST_CUDA(cudaStreamSynchronize(cst));
    return AST_OK;
}

int ast_step_host(ast_solver* S, const double* s_in, const double* u_in, double* s_out, double* u_out)
{
    // one step reads only the first pair
    return host_steps(S, 1, const_cast<double*>(s_in), const_cast<double*>(u_in), s_out, u_out);
}

int ast_step_host_n(ast_solver* S, int nsteps, double* s_a, double* u_a, double* s_b, double* u_b)
{
    return host_steps(S, nsteps, s_a, u_a, s_b, u_b);
}

int ast_synchronize(ast_solver* S)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    AST_CUDA(cudaStreamSynchronize(S->stream));
    unsigned int status = 0;
    AST_CUDA(cudaMemcpy(&status, &S->clock->status, sizeof status, cudaMemcpyDeviceToHost));
    if (status & AST_ST_NONFINITE) return fail(AST_ERR_NUMERIC, "non-finite wave speed");
    if (status & AST_ST_TIMEOUT) return fail(AST_ERR_CUDA, "a bulk tile copy did not arrive in time");
    return AST_OK;
}

int ast_get_phase_clocks(ast_solver* S, uint64_t out[8], int reset)
{
    if (!S || !out) return fail(AST_ERR_INVALID, "null argument");
#ifdef AST_PHASE_CLOCKS
    DevClock c;
    AST_CUDA(cudaMemcpyAsync(&c, S->clock, sizeof c, cudaMemcpyDeviceToHost, S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    for (int i = 0; i < 8; i++) out[i] = c.phase[i];
    if (reset) {
        std::memset(c.phase, 0, sizeof c.phase);
        AST_CUDA(cudaMemcpyAsync(S->clock, &c, sizeof c, cudaMemcpyHostToDevice, S->stream));
        AST_CUDA(cudaStreamSynchronize(S->stream));
    }
    return AST_OK;
#else
    (void)reset;
    return fail(AST_ERR_UNSUPPORTED, "the library was built without AST_PHASE_CLOCKS");
#endif
}

int ast_get_stats(ast_solver* S, ast_stats* out, int reset)
{
    if (!S || !out) return fail(AST_ERR_INVALID, "null argument");
    DevClock c;
    AST_CUDA(cudaMemcpyAsync(&c, S->clock, sizeof c, cudaMemcpyDeviceToHost, S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    std::memset(out, 0, sizeof *out);
    out->status = c.status;
    out->rho_floor = c.cnt[0];
    out->p_floor = c.cnt[1];
    out->newton_calls = c.cnt[2];
    out->newton_iters = c.cnt[3];
    out->bisect_calls = c.cnt[4];
    out->bisect_iters = c.cnt[5];
    out->mlp_fallback = c.cnt[6];
    out->newton_max_iters = (uint32_t)c.cnt[7];
    out->strong_calls = c.cnt[8];
    out->strong_iters = c.cnt[9];
    if (reset) {
        c.status = 0;
        std::memset(c.cnt, 0, sizeof c.cnt);
        AST_CUDA(cudaMemcpyAsync(S->clock, &c, sizeof c, cudaMemcpyHostToDevice, S->stream));
        AST_CUDA(cudaStreamSynchronize(S->stream));
    }
    return AST_OK;
}

static void drop_graph(ast_solver* S)
{
    if (S->graph) {
        cudaGraphExecDestroy(S->graph);
        S->graph = nullptr;
    }
}

int ast_set_mlp(ast_solver* S, const float* params)
{
    if (!S || !params) return fail(AST_ERR_INVALID, "null argument");
    // the parameter block and, after it, its packed form for the step kernels
    if (!S->mlp) AST_CUDA(cudaMalloc(&S->mlp, sizeof(float) * kMlpDevFloats));
    AST_CUDA(cudaMemcpyAsync(S->mlp, params, sizeof(float) * AST_MLP_NPARAM, cudaMemcpyHostToDevice, S->stream));
    const int rc = launch_mlp_pack(S->mlp, S->stream);
    if (rc != AST_OK) return rc;
    AST_CUDA(cudaStreamSynchronize(S->stream));
    S->P.mlp = S->mlp;
    drop_graph(S);
    return AST_OK;
}

int ast_set_neutral(ast_solver* S, const double* nn2, int on_device)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    drop_graph(S);   // captured steps hold the old parameters
    if (!nn2) {
        S->P.nsrc = nullptr;
        return AST_OK;
    }
    const long long K = (long long)S->cfg.N * S->cfg.M;
    if (!S->nsrc) AST_CUDA(cudaMalloc(&S->nsrc, (size_t)S->plane * 2 * S->elem));
    const double* src = nn2;
    double* tmp = nullptr;
    if (!on_device) {
        AST_CUDA(cudaMalloc(&tmp, (size_t)K * 3 * sizeof(double)));
        cudaError_t e = cudaMemcpyAsync(tmp, nn2, (size_t)K * 3 * sizeof(double), cudaMemcpyHostToDevice, S->stream);
        if (e != cudaSuccess) {
            cudaFree(tmp);
            return cuda_fail(e, "cudaMemcpyAsync nn2");
        }
        src = tmp;
    }
    const int nb = (int)((K + 255) / 256);
    if (S->elem == 8)
        nn2_to_planes<double><<<nb, 256, 0, S->stream>>>(src, (double*)S->nsrc, S->cfg.N, S->cfg.M, S->ld, S->plane);
    else
        nn2_to_planes<float><<<nb, 256, 0, S->stream>>>(src, (float*)S->nsrc, S->cfg.N, S->cfg.M, S->ld, S->plane);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(S->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return cuda_fail(e, "neutral source conversion");
    S->P.nsrc = S->nsrc;
    return AST_OK;
}

int ast_set_scalar(ast_solver* S, const double* q, int on_device)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    drop_graph(S);   // captured steps do not hold the scalar's launches
    if (!q) {
        S->has_q = false;
        return AST_OK;
    }
    if (S->elem != 8) return fail(AST_ERR_UNSUPPORTED, "the passive scalar is carried by the FP64 solver");
    if (S->cfg.flux != AST_FLUX_HLLC && S->cfg.flux != AST_FLUX_HLLCQ)
        return fail(AST_ERR_UNSUPPORTED, "the passive scalar needs the HLLC or HLLCQ flux");
    if (S->cfg.region_select) return fail(AST_ERR_UNSUPPORTED, "the passive scalar has no first-order region");
    const size_t bytes = (size_t)S->cfg.N * S->cfg.M * sizeof(double);
    for (int i = 0; i < 2; i++)
        if (!S->q[i]) AST_CUDA(cudaMalloc(&S->q[i], bytes));
    AST_CUDA(cudaMemcpyAsync(S->q[S->cur], q, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    S->has_q = true;
    return AST_OK;
}

int ast_get_scalar(ast_solver* S, double* q, int on_device)
{
    if (!S || !q) return fail(AST_ERR_INVALID, "null argument");
    if (!S->has_q) return fail(AST_ERR_INVALID, "no passive scalar set");
    const size_t bytes = (size_t)S->cfg.N * S->cfg.M * sizeof(double);
    AST_CUDA(cudaMemcpyAsync(q, S->q[S->cur], bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    return AST_OK;
}

int ast_probe(ast_solver* S, const int64_t* cells, int n, double* rho, double* TT)
{
    if (!S || n < 0 || (n > 0 && (!cells || !rho))) return fail(AST_ERR_INVALID, "bad argument");
    const long long K = (long long)S->cfg.N * S->cfg.M;
    for (int i = 0; i < n; i++)
        if (cells[i] < 0 || cells[i] >= K) return fail(AST_ERR_INVALID, "probe cell outside the grid");
    if (n > S->probe_cap) {
        cudaFree(S->probe_buf);
        S->probe_buf = nullptr;
        S->probe_cap = 0;
        AST_CUDA(cudaMalloc(&S->probe_buf, (size_t)n * 16));
        S->probe_cap = n;
    }
    if (n > 0) {
        double* dout = reinterpret_cast<double*>(S->probe_buf + n);
        AST_CUDA(cudaMemcpyAsync(S->probe_buf, cells, (size_t)n * 8, cudaMemcpyHostToDevice, S->stream));
        const void* q = S->buf[S->cur];
        if (S->elem == 8)
            probe_kernel<double><<<(n + 127) / 128, 128, 0, S->stream>>>((const double*)q, S->ld, S->cfg.N, S->probe_buf,
                                                                        n, dout);
        else
            probe_kernel<float><<<(n + 127) / 128, 128, 0, S->stream>>>((const float*)q, S->ld, S->cfg.N, S->probe_buf,
                                                                       n, dout);
        AST_CUDA(cudaGetLastError());
        AST_CUDA(cudaMemcpyAsync(rho, dout, (size_t)n * 8, cudaMemcpyDeviceToHost, S->stream));
    }
    if (TT) AST_CUDA(cudaMemcpyAsync(TT, &S->clock->TT, sizeof(double), cudaMemcpyDeviceToHost, S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    return AST_OK;
}

int ast_record_start(ast_solver* S, int64_t capacity, int every, double min_strength)
{
    if (!S || capacity < 1 || every < 1) return fail(AST_ERR_INVALID, "bad argument");
    if (S->cfg.flux != AST_FLUX_GODUNOV) return fail(AST_ERR_UNSUPPORTED, "the recorder needs the exact solver");
    if (S->cfg.precision != AST_PREC_FP64) return fail(AST_ERR_UNSUPPORTED, "the recorder runs on the FP64 solver");
    cudaFree(S->rec);
    S->rec = nullptr;
    if (!S->rec_n) AST_CUDA(cudaMalloc(&S->rec_n, sizeof(unsigned long long)));
    cudaError_t e = cudaMalloc(&S->rec, sizeof(float) * AST_RECORD_FLOATS * (size_t)capacity);
    if (e != cudaSuccess) return fail(AST_ERR_NOMEM, "recorder buffer");
    AST_CUDA(cudaMemsetAsync(S->rec_n, 0, sizeof(unsigned long long), S->stream));
    S->rec_cap = capacity;
    S->P.rec = S->rec;
    S->P.rec_n = S->rec_n;
    S->P.rec_cap = capacity;
    S->P.rec_every = every;
    S->P.rec_gate = min_strength;
    drop_graph(S);
    return AST_OK;
}

int ast_record_stop(ast_solver* S, int64_t* offered)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    unsigned long long n = 0;
    if (S->rec_n) {
        AST_CUDA(cudaMemcpyAsync(&n, S->rec_n, sizeof n, cudaMemcpyDeviceToHost, S->stream));
        AST_CUDA(cudaStreamSynchronize(S->stream));
    }
    if (offered) *offered = (int64_t)n;
    S->P.rec = nullptr;
    drop_graph(S);
    return AST_OK;
}

int ast_record_read(ast_solver* S, float* out, int64_t n)
{
    if (!S || !out || n < 0) return fail(AST_ERR_INVALID, "bad argument");
    if (!S->rec) return fail(AST_ERR_INVALID, "no recorder buffer");
    n = n < S->rec_cap ? n : S->rec_cap;
    AST_CUDA(cudaMemcpyAsync(out, S->rec, sizeof(float) * AST_RECORD_FLOATS * (size_t)n, cudaMemcpyDeviceToHost,
                             S->stream));
    AST_CUDA(cudaStreamSynchronize(S->stream));
    return AST_OK;
}

int ast_device_state(ast_solver* S, void** planes, int64_t* ld, int* elem_bytes)
{
    if (!S) return fail(AST_ERR_INVALID, "null solver");
    if (planes) *planes = S->buf[S->cur];
    if (ld) *ld = S->ld;
    if (elem_bytes) *elem_bytes = (int)S->elem;
    return AST_OK;
}

// ==================================================================== kernel-level drop-in
static int step_raw(const double* s, const double* u, double* s2, double* u2, const double* nn2, double* T,
                    const double* T_do, const ast_config* cfg, void* stream)
{
    if (!s || !u || !s2 || !u2 || !T || !T_do || !cfg) return fail(AST_ERR_INVALID, "null argument");
    int rc = ast_config_check(cfg);
    if (rc != AST_OK) return rc;
    if (cfg->precision != AST_PREC_FP64) return fail(AST_ERR_UNSUPPORTED, "raw step is FP64 (reference layout)");
    if (cfg->guess == AST_GUESS_MLP) return fail(AST_ERR_UNSUPPORTED, "raw step has no learned start value");
    StepParams P;
    fill_step_params(P, *cfg);
    P.in = s;
    P.in_u = u;
    P.out = s2;
    P.out_u = u2;
    P.clock = nullptr;
    P.T_min = T;
    P.T_do_ptr = T_do;
    P.collect_stats = 0;
    P.nsrc = nn2;
    rc = launch_step_r<double, kAoS>(P, cfg->flux, cfg->recon, (cudaStream_t)stream, false);
    if (rc != AST_OK) return rc;
    return launch_step_r<double, kAoS>(P, cfg->flux, cfg->recon, (cudaStream_t)stream, true);
}

int ast_step_raw(const double* s, const double* u, double* s2, double* u2, double* T, const double* T_do,
                 const double* TT, int method, const ast_config* cfg, void* stream)
{
    (void)TT;
    (void)method;
    return step_raw(s, u, s2, u2, nullptr, T, T_do, cfg, stream);
}

int ast_add_mk_raw(const double* s, const double* u, double* s2, double* u2, const double* nn1, const double* nn2,
                   const double* nn3, double* T, const double* T_do, int method, int step, const ast_config* cfg,
                   void* stream)
{
    (void)nn1;
    (void)nn3;
    (void)method;
    (void)step;
    return step_raw(s, u, s2, u2, nn2, T, T_do, cfg, stream);
}

int ast_inflow_raw(const double* s, const double* u, double* s2, double* u2, const ast_config* cfg, void* stream)
{
    if (!s || !u || !s2 || !u2 || !cfg) return fail(AST_ERR_INVALID, "null argument");
    int rc = ast_config_check(cfg);
    if (rc != AST_OK) return rc;
    if (!(cfg->inflow_p > 0.0)) return fail(AST_ERR_INVALID, "inflow_p must be positive");
    StepParams P;
    fill_step_params(P, *cfg);
    P.in = s;
    P.in_u = u;
    P.out = s2;
    P.out_u = u2;
    inflow_kernel<double, kAoS><<<(cfg->M + 127) / 128, 128, 0, (cudaStream_t)stream>>>(P, cfg->inflow_p,
                                                                                       cfg->inflow_v);
    AST_CUDA(cudaGetLastError());
    return AST_OK;
}

int ast_funk_time(double* T, double* T_do, double* TT, int* i, void* stream)
{
    if (!T || !T_do || !TT || !i) return fail(AST_ERR_INVALID, "null argument");
    funk_time_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(T, T_do, TT, i);
    AST_CUDA(cudaGetLastError());
    return AST_OK;
}

}  // extern "C"
