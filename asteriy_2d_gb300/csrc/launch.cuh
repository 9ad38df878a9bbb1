// launch.cuh - launch helpers of the step kernel.  The instantiations are
// spread over several translation units (step_f64.cu, step_f32.cu,
// step_raw.cu) so that they compile in parallel.
#pragma once

#include <cuda_runtime.h>

#include "../../include/asteriy_gb300.h"
#include "step.cuh"

namespace ast {

constexpr int kTZ = 32, kTR = 16;

// records the failure text for ast_last_error() and returns AST_ERR_CUDA
int cuda_fail(cudaError_t e, const char* what);

// launch=false only raises the kernel's dynamic shared-memory limit, which
// must happen outside stream capture (ast_create, ast_step_raw)
template <typename R, int FLUX, bool RECON, int LAYOUT>
int launch_step_t(const StepParams& P, cudaStream_t st, bool launch)
{
    auto k = step_kernel<R, FLUX, RECON, LAYOUT, kTZ, kTR>;
    constexpr size_t smem = tile_smem_bytes<R, kTZ, kTR>();
    cudaError_t e;
    if (!launch) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return e == cudaSuccess ? AST_OK : cuda_fail(e, "cudaFuncSetAttribute");
    }
    dim3 grid((P.N + kTZ - 1) / kTZ, (P.M + kTR - 1) / kTR);
    k<<<grid, kThreads, smem, st>>>(P);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "step kernel launch");
}

template <typename R, int LAYOUT>
int launch_step_r(const StepParams& P, int flux, int recon, cudaStream_t st, bool launch)
{
    if (recon) {
        if (flux == AST_FLUX_HLL) return launch_step_t<R, 0, true, LAYOUT>(P, st, launch);
        if (flux == AST_FLUX_HLLC) return launch_step_t<R, 1, true, LAYOUT>(P, st, launch);
        return launch_step_t<R, 2, true, LAYOUT>(P, st, launch);
    }
    if (flux == AST_FLUX_HLL) return launch_step_t<R, 0, false, LAYOUT>(P, st, launch);
    if (flux == AST_FLUX_HLLC) return launch_step_t<R, 1, false, LAYOUT>(P, st, launch);
    return launch_step_t<R, 2, false, LAYOUT>(P, st, launch);
}

extern template int launch_step_r<double, kSoA>(const StepParams&, int, int, cudaStream_t, bool);
extern template int launch_step_r<float, kSoA>(const StepParams&, int, int, cudaStream_t, bool);
extern template int launch_step_r<double, kAoS>(const StepParams&, int, int, cudaStream_t, bool);

}  // namespace ast
