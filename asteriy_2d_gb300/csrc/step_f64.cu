// step_f64.cu - step kernel instantiations for FP64 state planes (solver path):
// one CTA per tile, and the persistent kernel.
#include "launch.cuh"

namespace ast {
template int launch_step_r<double, kSoA>(const StepParams&, int, int, cudaStream_t, bool);

int launch_step_tma64(const StepParams& P, const CUtensorMap& tin, const CUtensorMap& tout, int flux, int recon,
                      int grid, cudaStream_t st, bool launch, int* per_sm)
{
#define AST_TMA64(F, RC) return launch_tma_t<double, F, RC>(P, tin, tout, grid, st, launch, per_sm)
    if (recon) {
        if (flux == AST_FLUX_HLL) AST_TMA64(0, true);
        if (flux == AST_FLUX_HLLC) AST_TMA64(1, true);
        if (flux == AST_FLUX_HLLC_A) AST_TMA64(3, true);
        if (flux == AST_FLUX_HLLCQ) AST_TMA64(4, true);
        AST_TMA64(2, true);
    }
    if (flux == AST_FLUX_HLL) AST_TMA64(0, false);
    if (flux == AST_FLUX_HLLC) AST_TMA64(1, false);
    if (flux == AST_FLUX_HLLC_A) AST_TMA64(3, false);
    if (flux == AST_FLUX_HLLCQ) AST_TMA64(4, false);
    AST_TMA64(2, false);
#undef AST_TMA64
}
}  // namespace ast
