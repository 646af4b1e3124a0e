// Persistent mixed-batch kernels for the scmos camera family; see gmle_mixed.cuh.
#include "gmle_mixed.cuh"

namespace gmle {

namespace {

using KernelFn = void (*)(const MixedArgs);

KernelFn kernel_of(int cls)
{
    return cls == 0 ? fit_mixed_kernel<true, 0>
                    : (cls == 1 ? fit_mixed_kernel<true, 1> : fit_mixed_kernel<true, 2>);
}

bool attr_done[3] = {false, false, false};

cudaError_t ensure_attr(int cls)
{
    if (attr_done[cls]) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(kernel_of(cls),
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, kMixedMaxSmem);
    if (e == cudaSuccess) attr_done[cls] = true;
    return e;
}

}  // namespace

cudaError_t launch_mixed_scmos(int cls, const MixedArgs &m, size_t smem, int grid, cudaStream_t s)
{
    if (cls < 0 || cls > 2) return cudaErrorInvalidValue;
    cudaError_t e = ensure_attr(cls);
    if (e != cudaSuccess) return e;
    kernel_of(cls)<<<grid, m.rois_per_tile, smem, s>>>(m);
    return cudaGetLastError();
}

int mixed_blocks_per_sm_scmos(int cls, size_t smem)
{
    if (cls < 0 || cls > 2 || ensure_attr(cls) != cudaSuccess) return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel_of(cls), class_tile(cls), smem) !=
        cudaSuccess)
        return 0;
    return nb;
}

cudaError_t mixed_set_attributes_scmos()
{
    for (int c = 0; c < 3; c++) {
        cudaError_t e = cudaFuncSetAttribute(kernel_of(c), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kMixedMaxSmem);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace gmle
