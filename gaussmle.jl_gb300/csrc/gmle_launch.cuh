// gmle_launch.cuh - launch of one fit-kernel specialisation.  Each
// gmle_fit_<model>.cu translation unit instantiates the kernels of one PSF
// model for every supported box size and camera family, so the four units
// compile in parallel.
#pragma once

#include "gmle_fit_kernel.cuh"

namespace gmle {

// Box sizes with a compiled specialisation (the configurations use 7..15).
constexpr int kBoxes[] = {5, 7, 9, 11, 13, 15};

inline bool box_supported(int box)
{
    for (int b : kBoxes)
        if (b == box) return true;
    return false;
}

cudaError_t launch_fit_model0(int box, bool scmos, const KernelArgs &a, int rois_per_block,
                              cudaStream_t s);
cudaError_t launch_fit_model1(int box, bool scmos, const KernelArgs &a, int rois_per_block,
                              cudaStream_t s);
cudaError_t launch_fit_model2(int box, bool scmos, const KernelArgs &a, int rois_per_block,
                              cudaStream_t s);
cudaError_t launch_fit_model3(int box, bool scmos, const KernelArgs &a, int rois_per_block,
                              cudaStream_t s);

template <int MODEL, int BOX, bool SCMOS>
cudaError_t launch_one(const KernelArgs &a, int rois_per_block, cudaStream_t s)
{
    const int threads = rois_per_block * a.tpr;
    const size_t smem = smem_bytes(MODEL, BOX, SCMOS, a.tpr, rois_per_block);
    static bool attr_done = false;  // per specialisation; set once per process
    if (!attr_done) {
        cudaError_t e = cudaFuncSetAttribute(fit_kernel<MODEL, BOX, SCMOS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             227 * 1024);
        if (e != cudaSuccess) return e;
        attr_done = true;
    }
    const int64_t blocks = (a.n + rois_per_block - 1) / rois_per_block;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    fit_kernel<MODEL, BOX, SCMOS><<<(unsigned)blocks, threads, smem, s>>>(a);
    return cudaGetLastError();
}

template <int MODEL>
cudaError_t launch_model(int box, bool scmos, const KernelArgs &a, int rois_per_block,
                         cudaStream_t s)
{
#define GMLE_CASE(B)                                                                     \
    case B:                                                                              \
        return scmos ? launch_one<MODEL, B, true>(a, rois_per_block, s)                  \
                     : launch_one<MODEL, B, false>(a, rois_per_block, s);
    switch (box) {
        GMLE_CASE(5)
        GMLE_CASE(7)
        GMLE_CASE(9)
        GMLE_CASE(11)
        GMLE_CASE(13)
        GMLE_CASE(15)
        default:
            return cudaErrorInvalidValue;
    }
#undef GMLE_CASE
}

}  // namespace gmle
