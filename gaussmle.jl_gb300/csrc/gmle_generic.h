// gmle_generic.h - launch of the run-time-box fit kernel (gmle_fit_generic.cu)
// for the boxes the specialised kernels do not take.
#pragma once

#include <cuda_runtime.h>

#include "gmle_fit_kernel.cuh"

namespace gmle {

constexpr int kGenericMinBox = 17, kGenericMaxBox = 64;

inline bool generic_box(int box) { return box >= kGenericMinBox && box <= kGenericMaxBox; }

// ROIs per block of the run-time-box kernel (one thread each).
int generic_rois_per_block(int box, bool scmos);

// Plain launch of ceil(a.n / rois per block) blocks over `a` (a.tpr == 1).
cudaError_t launch_fit_generic(int model, int box, bool scmos, const KernelArgs &a, cudaStream_t s);

}  // namespace gmle
