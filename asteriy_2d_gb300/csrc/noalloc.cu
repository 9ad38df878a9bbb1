// noalloc.cu - a step with the dt shift (Kernel_TVD + funk_time) that
// allocates nothing.
//
// Who needs it: code that must not call cudaMalloc while it steps - a
// process whose device memory is carved up by a different allocator under a
// fixed budget, or a real-time loop where an allocation's latency or failure
// is not acceptable.  ast_step_raw already needs no scratch, but it leaves
// the dt shift to a second call (ast_funk_time); the solver object shifts dt
// inside its step kernel but owns device memory that ast_create allocates.
// This entry point does the step and the shift on the caller's
// reference-layout arrays with the cross-CTA reduction state (the device
// clock: wave-speed maxima, CTA ticket, status, counters) in a file-scope
// device array instead of allocated memory.  It enqueues three kernels on
// the caller's stream: a one-thread kernel that clears the array and copies
// T_do, TT and step in, the step kernel, and a one-thread kernel that copies
// the shifted T_do, TT and step (and the status bits) back out.
//
// Limits and sharing:
//   - the scratch is a fixed AST_NOALLOC_SCRATCH_BYTES block per device,
//     held from library load until process exit; it does not grow with the
//     grid, so every grid that ast_config_check accepts fits;
//   - every call shares the block and it keeps the last call's contents:
//     each call clears all of it first; calls that overlap on the GPU
//     (other streams, other host threads) race on it and must be serialised
//     by the caller;
//   - the first call on a device looks up the block's device address
//     (cudaGetSymbolAddress) and raises the kernel's shared-memory limit;
//     make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/asteriy_gb300.h"
#include "launch.cuh"

using namespace ast;

namespace {

static_assert(sizeof(DevClock) <= AST_NOALLOC_SCRATCH_BYTES, "device clock must fit the static scratch");

// the scratch; host code must not use this name as an address
static __device__ __align__(256) unsigned char g_step_scratch[AST_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
DevClock* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_setup_mu;

// clock in: every field cleared, then T_do / TT / step taken from the caller
__global__ void clock_in(DevClock* C, const double* T_do, const double* TT, const int64_t* step)
{
    C->T_do = *T_do;
    C->TT = *TT;
    C->step = (long long)*step;
    C->smax_z = 0ull;
    C->smax_r = 0ull;
    C->done = 0u;
    C->status = 0u;
    for (int i = 0; i < (int)(sizeof(C->cnt) / sizeof(C->cnt[0])); i++) C->cnt[i] = 0ull;
    C->next_tile = 0u;
    C->pad_ = 0u;
    C->T_prev = 0.0;
}

// clock out: the shifted T_do, TT and step back to the caller
__global__ void clock_out(const DevClock* C, double* T_do, double* TT, int64_t* step, unsigned int* status)
{
    *T_do = C->T_do;
    *TT = C->TT;
    *step = (int64_t)C->step;
    if (status) *status = C->status;
}

int scratch_for_current_device(DevClock** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return AST_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_step_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
        StepParams none{};
        int rc = launch_step_r<double, kAoS>(none, AST_FLUX_HLL, 0, nullptr, false);
        for (int f = AST_FLUX_HLL; rc == AST_OK && f <= AST_FLUX_GODUNOV; f++)
            for (int r = 0; rc == AST_OK && r <= 1; r++) rc = launch_step_r<double, kAoS>(none, f, r, nullptr, false);
        if (rc != AST_OK) return rc;
        g_scratch_ptr[dev] = (DevClock*)p;
    }
    *out = g_scratch_ptr[dev];
    return AST_OK;
}

}  // namespace

extern "C" int ast_step_noalloc(const double* s, const double* u, double* s2, double* u2, double* T_do, double* TT,
                                int64_t* step, unsigned int* status, const ast_config* cfg, void* stream)
{
    if (!s || !u || !s2 || !u2 || !T_do || !TT || !step || !cfg) return AST_ERR_INVALID;
    int rc = ast_config_check(cfg);
    if (rc != AST_OK) return rc;
    if (cfg->precision != AST_PREC_FP64 || cfg->guess == AST_GUESS_MLP) return AST_ERR_UNSUPPORTED;
    DevClock* C = nullptr;
    rc = scratch_for_current_device(&C);
    if (rc != AST_OK) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    StepParams P;
    fill_step_params(P, *cfg);
    P.in = s;
    P.in_u = u;
    P.out = s2;
    P.out_u = u2;
    P.clock = C;
    P.collect_stats = 0;
    clock_in<<<1, 1, 0, st>>>(C, T_do, TT, step);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "clock_in launch");
    rc = launch_step_r<double, kAoS>(P, cfg->flux, cfg->recon, st, true);
    if (rc != AST_OK) return rc;
    clock_out<<<1, 1, 0, st>>>(C, T_do, TT, step, status);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "clock_out launch");
}
