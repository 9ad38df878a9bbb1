// batch_mixed.cu - the FP32 batch kernels over problems of every flux in
// one launch (32x16 tiles): a CTA per tile, and the persistent kernel.
#include "launch.cuh"

namespace ast {

template <bool RECON>
static int launch_mixed_t(const StepParams* Ps, const int* tile_start, const int* flux_of, int nprob, int tiles,
                          cudaStream_t st, bool launch)
{
    constexpr int TZ = kShapeTZ[0], TR = kShapeTR[0];
    auto k = batch_kernel_mixed<float, RECON, TZ, TR>;
    constexpr size_t smem =
        std::max(std::max(tile_smem_bytes<float, 0, TZ, TR>(), tile_smem_bytes<float, 1, TZ, TR>()),
                 std::max(tile_smem_bytes<float, 2, TZ, TR>(), tile_smem_bytes<float, 3, TZ, TR>()));
    cudaError_t e;
    if (!launch) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        return e == cudaSuccess ? AST_OK : cuda_fail(e, "cudaFuncSetAttribute");
    }
    if (tiles <= 0) return AST_OK;
    k<<<tiles, kThreads, smem, st>>>(Ps, tile_start, flux_of, nprob);
    e = cudaGetLastError();
    return e == cudaSuccess ? AST_OK : cuda_fail(e, "mixed batch kernel launch");
}

int launch_batch_mixed(const StepParams* Ps, const int* tile_start, const int* flux_of, int nprob, int tiles,
                       int recon, cudaStream_t st, bool launch)
{
    return recon ? launch_mixed_t<true>(Ps, tile_start, flux_of, nprob, tiles, st, launch)
                 : launch_mixed_t<false>(Ps, tile_start, flux_of, nprob, tiles, st, launch);
}

int launch_batch_tma_mixed(const StepParams* Ps, const CUtensorMap* tin, const CUtensorMap* tout,
                           const BatchTile* work, int total, int nslots, unsigned int* counter, int wait_polls,
                           int recon, int grid, cudaStream_t st, bool launch, int* per_sm)
{
    return recon ? launch_batch_tma_t<2, true, true>(Ps, tin, tout, work, total, 0, nslots, counter, wait_polls,
                                                     grid, st, launch, per_sm)
                 : launch_batch_tma_t<2, false, true>(Ps, tin, tout, work, total, 0, nslots, counter, wait_polls,
                                                      grid, st, launch, per_sm);
}

}  // namespace ast
