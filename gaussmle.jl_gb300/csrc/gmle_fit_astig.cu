// Fit-kernel specialisations for PSF model 3 (astig); see gmle_launch.cuh.
#include "gmle_launch.cuh"

namespace gmle {
cudaError_t launch_fit_model3(int box, bool scmos, const KernelArgs &a, int rois_per_block,
                              cudaStream_t s)
{
    return launch_model<3>(box, scmos, a, rois_per_block, s);
}
}  // namespace gmle
