// Persistent mixed-batch kernel for the scmos camera family; see gmle_mixed.cuh.
#include "gmle_mixed.cuh"

namespace gmle {

static bool attr_done = false;

static cudaError_t ensure_attr()
{
    if (attr_done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(fit_mixed_kernel<true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kMixedMaxSmem);
    if (e == cudaSuccess) attr_done = true;
    return e;
}

cudaError_t launch_mixed_scmos(const MixedArgs &m, size_t smem, int grid, cudaStream_t s)
{
    cudaError_t e = ensure_attr();
    if (e != cudaSuccess) return e;
    fit_mixed_kernel<true><<<grid, m.rois_per_tile, smem, s>>>(m);
    return cudaGetLastError();
}

int mixed_blocks_per_sm_scmos(size_t smem)
{
    int nb = 0;
    if (ensure_attr() != cudaSuccess) return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fit_mixed_kernel<true>, 32, smem) !=
        cudaSuccess)
        return 0;
    return nb;
}

}  // namespace gmle
