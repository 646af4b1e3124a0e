// gmle_fit_family.cu - the fit kernels of one part of one PSF model and
// camera family (gmle_launch.cuh).  Compiled once per (model, camera family,
// part) with -DGMLE_MODEL=0..3 -DGMLE_SCMOS=0|1 -DGMLE_PART=0..2, so that the
// parts compile in parallel; each unit explicitly instantiates its part's
// launch and residency functions, which the runtime reaches through the
// extern template declarations of gmle_launch.cuh.
#if !defined(GMLE_MODEL) || !defined(GMLE_SCMOS) || !defined(GMLE_PART)
#error "compile with -DGMLE_MODEL=<0..3> -DGMLE_SCMOS=<0|1> -DGMLE_PART=<0..2>"
#endif

#include "gmle_launch.cuh"

namespace gmle {
template cudaError_t launch_part<GMLE_MODEL, (GMLE_SCMOS != 0), GMLE_PART>(
    int, const KernelArgs &, const TileTable &, const LaunchShape &, cudaStream_t);
template int table_blocks_part<GMLE_MODEL, (GMLE_SCMOS != 0), GMLE_PART>(int, int, int);
}  // namespace gmle
