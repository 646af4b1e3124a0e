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

// Largest block of the one-thread-per-ROI kernel (its __launch_bounds__).
constexpr int kMaxThreadsR1 = 64;

template <int MODEL, int BOX, bool SCMOS>
cudaError_t launch_one(const KernelArgs &a, int rois_per_block, cudaStream_t s)
{
    const int threads = rois_per_block * a.tpr;
    const size_t smem = smem_bytes(MODEL, BOX, SCMOS, a.tpr, rois_per_block);
    const bool r1 = a.tpr == 1;
    if (r1 && threads > kMaxThreadsR1) return cudaErrorInvalidConfiguration;
    void (*kern)(const KernelArgs) = r1 ? fit_kernel_r1<MODEL, BOX, SCMOS>
                                        : fit_kernel<MODEL, BOX, SCMOS>;
    static bool attr_done[2] = {false, false};  // per specialisation and kernel
    if (!attr_done[r1]) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             227 * 1024);
        if (e != cudaSuccess) return e;
        attr_done[r1] = true;
    }
    const int64_t blocks = (a.n + rois_per_block - 1) / rois_per_block;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    kern<<<(unsigned)blocks, threads, smem, s>>>(a);
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
