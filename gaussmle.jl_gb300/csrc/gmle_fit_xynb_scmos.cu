// Fit-kernel specialisations for PSF model 0 (GaussianXYNB), sCMOS camera;
// see gmle_launch.cuh.
#include "gmle_launch.cuh"

namespace gmle {
cudaError_t launch_fit_m0_scmos(int box, const KernelArgs &a, const TileTable &t,
                                const LaunchShape &shape, cudaStream_t s)
{
    return launch_family<0, true>(box, a, t, shape, s);
}
int table_blocks_m0_scmos(int box, int tpr, int rois_per_block)
{
    return table_blocks_family<0, true>(box, tpr, rois_per_block);
}
}  // namespace gmle
