// Fit-kernel specialisations for PSF model 2 (GaussianXYNBSXSY), Poisson (IdealCamera) camera;
// see gmle_launch.cuh.
#include "gmle_launch.cuh"

namespace gmle {
cudaError_t launch_fit_m2_poisson(int box, const KernelArgs &a, const TileTable &t,
                                const LaunchShape &shape, cudaStream_t s)
{
    return launch_family<2, false>(box, a, t, shape, s);
}
int table_blocks_m2_poisson(int box, int tpr, int rois_per_block)
{
    return table_blocks_family<2, false>(box, tpr, rois_per_block);
}
}  // namespace gmle
