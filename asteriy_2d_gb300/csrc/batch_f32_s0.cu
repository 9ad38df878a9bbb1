// batch_f32_s0.cu - batch kernel instantiations, FP32 state planes, tile shape 0.
#include "launch.cuh"

namespace ast {
int launch_batch_tma(const StepParams* Ps, const CUtensorMap* tin, const CUtensorMap* tout, const BatchTile* work,
                     int total, int slot0, int nslots, unsigned int* counter, int wait_polls, int flux, int recon,
                     int grid, cudaStream_t st, bool launch, int* per_sm)
{
#define AST_BTMA(F, RC)                                                                                            \
    return launch_batch_tma_t<F, RC, false>(Ps, tin, tout, work, total, slot0, nslots, counter, wait_polls, grid, \
                                            st, launch, per_sm)
    if (recon) {
        if (flux == AST_FLUX_HLL) AST_BTMA(0, true);
        if (flux == AST_FLUX_HLLC) AST_BTMA(1, true);
        if (flux == AST_FLUX_HLLC_A) AST_BTMA(3, true);
        AST_BTMA(2, true);
    }
    if (flux == AST_FLUX_HLL) AST_BTMA(0, false);
    if (flux == AST_FLUX_HLLC) AST_BTMA(1, false);
    if (flux == AST_FLUX_HLLC_A) AST_BTMA(3, false);
    AST_BTMA(2, false);
#undef AST_BTMA
}

template int launch_batch_r<float, kShapeTZ[0], kShapeTR[0]>(const StepParams*, const int*, int, int, int, int,
                                                            cudaStream_t, bool);
}  // namespace ast
