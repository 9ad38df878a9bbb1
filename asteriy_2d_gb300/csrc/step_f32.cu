// step_f32.cu - step kernel instantiations for FP32 state planes (precision form).
#include "launch.cuh"

namespace ast {
template int launch_step_r<float, kSoA>(const StepParams&, int, int, cudaStream_t, bool);

int launch_step_tma(const StepParams& P, const CUtensorMap& tin, const CUtensorMap& tout, int flux, int recon,
                    int grid, cudaStream_t st, bool launch, int* per_sm)
{
    if (recon) {
        if (flux == AST_FLUX_HLL) return launch_tma_t<float, 0, true>(P, tin, tout, grid, st, launch, per_sm);
        if (flux == AST_FLUX_HLLC) return launch_tma_t<float, 1, true>(P, tin, tout, grid, st, launch, per_sm);
        if (flux == AST_FLUX_HLLC_A) return launch_tma_t<float, 3, true>(P, tin, tout, grid, st, launch, per_sm);
        return launch_tma_t<float, 2, true>(P, tin, tout, grid, st, launch, per_sm);
    }
    if (flux == AST_FLUX_HLL) return launch_tma_t<float, 0, false>(P, tin, tout, grid, st, launch, per_sm);
    if (flux == AST_FLUX_HLLC) return launch_tma_t<float, 1, false>(P, tin, tout, grid, st, launch, per_sm);
    if (flux == AST_FLUX_HLLC_A) return launch_tma_t<float, 3, false>(P, tin, tout, grid, st, launch, per_sm);
    return launch_tma_t<float, 2, false>(P, tin, tout, grid, st, launch, per_sm);
}

int launch_step_sweep(const StepParams& P, int flux, int recon, int grid, cudaStream_t st, bool launch, int* per_sm)
{
    if (recon) {
        if (flux == AST_FLUX_HLL) return launch_sweep_t<0, true>(P, grid, st, launch, per_sm);
        if (flux == AST_FLUX_HLLC) return launch_sweep_t<1, true>(P, grid, st, launch, per_sm);
        if (flux == AST_FLUX_HLLC_A) return launch_sweep_t<3, true>(P, grid, st, launch, per_sm);
        return launch_sweep_t<2, true>(P, grid, st, launch, per_sm);
    }
    if (flux == AST_FLUX_HLL) return launch_sweep_t<0, false>(P, grid, st, launch, per_sm);
    if (flux == AST_FLUX_HLLC) return launch_sweep_t<1, false>(P, grid, st, launch, per_sm);
    if (flux == AST_FLUX_HLLC_A) return launch_sweep_t<3, false>(P, grid, st, launch, per_sm);
    return launch_sweep_t<2, false>(P, grid, st, launch, per_sm);
}
}  // namespace ast
