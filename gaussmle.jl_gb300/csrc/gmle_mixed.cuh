// gmle_mixed.cuh - persistent, work-stealing fit of a mixed batch in one launch.
//
// A mixed batch is a list of homogeneous groups (a serving request, or one
// (model, box) class of a heterogeneous batch), each with its own fit
// descriptor and device buffers.  The groups' ROIs are cut into tiles of
// `rois_per_tile` ROIs (a block of one-thread-per-ROI fits).  A persistent
// grid of CTAs pulls tile indices from a global atomic counter (work
// stealing), finds the tile's group and runs the fit specialised for the
// group's (model, box) on it; tiles of the most expensive groups come first
// so that the tail is short.  All four PSF models and every box of a
// shared-memory class share a launch; the camera family (Poisson or sCMOS)
// and the class are template parameters, so a batch takes one launch per
// (family, class) present, the classes of a family running concurrently.
#pragma once

#include "gmle_fit_kernel.cuh"

namespace gmle {

struct GroupDesc {
    const float *data;
    const int32_t *xc, *yc;
    int64_t n;
    float *params, *crlb, *llr;
    uint8_t *flags;
    int32_t model, box, iterations, adu;
    float psf[8], lower[6], upper[6], max_step[6];
    int64_t tile0;  // index of the group's first tile (groups sorted by tile0)
};

struct MixedArgs {
    const GroupDesc *groups;
    const int64_t *header;   // [0] = number of groups, [1] = number of tiles (device)
    unsigned long long *tile_counter;
    const float *var, *gain, *offset;
    int32_t ny, nx;
    int32_t rois_per_tile;   // = blockDim.x
    float sqrt2pi;
    unsigned long long *bad_corners;
};

// Boxes compiled into the mixed kernel.
__host__ __device__ constexpr bool mixed_box(int box)
{
    return box == 5 || box == 7 || box == 9 || box == 11 || box == 13 || box == 15;
}

template <int MODEL, int BOX, bool SCMOS>
__device__ __noinline__ void mixed_tile(const KernelArgs a, int64_t roi0, int nroi, float *smem)
{
    fit_rois_r1<MODEL, BOX, SCMOS>(a, roi0, nroi, smem);
}

// Shared-memory classes: ROIs up to 9x9, 11x11, and 13x13 or 15x15.  Each
// class has its own persistent kernel (so that its register allocation is
// that of its own box sizes) and tile size.
__host__ __device__ constexpr int box_class(int box) { return box <= 9 ? 0 : (box <= 11 ? 1 : 2); }
__host__ __device__ constexpr int class_tile(int cls) { return cls == 2 ? 32 : 64; }

template <bool SCMOS, int CLASS>
__device__ void mixed_dispatch(int model, int box, const KernelArgs &a, int64_t roi0, int nroi,
                               float *smem)
{
#define GMLE_MX(M, B) \
    case (M) * 32 + (B): mixed_tile<M, B, SCMOS>(a, roi0, nroi, smem); break;
    if (CLASS == 0) {
        switch (model * 32 + box) {
            GMLE_MX(0, 5) GMLE_MX(0, 7) GMLE_MX(0, 9) GMLE_MX(1, 5) GMLE_MX(1, 7) GMLE_MX(1, 9)
            GMLE_MX(2, 5) GMLE_MX(2, 7) GMLE_MX(2, 9) GMLE_MX(3, 5) GMLE_MX(3, 7) GMLE_MX(3, 9)
            default: break;
        }
    } else if (CLASS == 1) {
        switch (model * 32 + box) {
            GMLE_MX(0, 11) GMLE_MX(1, 11) GMLE_MX(2, 11) GMLE_MX(3, 11)
            default: break;
        }
    } else {
        switch (model * 32 + box) {
            GMLE_MX(0, 13) GMLE_MX(0, 15) GMLE_MX(1, 13) GMLE_MX(1, 15)
            GMLE_MX(2, 13) GMLE_MX(2, 15) GMLE_MX(3, 13) GMLE_MX(3, 15)
            default: break;
        }
    }
#undef GMLE_MX
}

template <bool SCMOS, int CLASS>
__global__ void __launch_bounds__(64) fit_mixed_kernel(const MixedArgs m)
{
    extern __shared__ __align__(16) float smem[];
    __shared__ long long s_tile;
    const int ngroups = (int)m.header[0];
    const long long ntiles = m.header[1];
    for (;;) {
        if (threadIdx.x == 0) s_tile = (long long)atomicAdd(m.tile_counter, 1ull);
        __syncthreads();
        const long long tile = s_tile;
        __syncthreads();  // all threads have read s_tile before it is rewritten
        if (tile >= ntiles) return;
        int lo = 0, hi = ngroups - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (m.groups[mid].tile0 <= tile) lo = mid; else hi = mid - 1;
        }
        const GroupDesc &G = m.groups[lo];
        KernelArgs a;
        a.data = G.data;
        a.xc = G.xc;
        a.yc = G.yc;
        a.n = G.n;
        a.var = m.var;
        a.gain = m.gain;
        a.offset = m.offset;
        a.ny = m.ny;
        a.nx = m.nx;
        a.adu = G.adu;
        a.iterations = G.iterations;
        a.tpr = 1;
        a.sqrt2pi = m.sqrt2pi;
#pragma unroll
        for (int t = 0; t < 8; t++) a.psf[t] = G.psf[t];
#pragma unroll
        for (int t = 0; t < 6; t++) {
            a.lower[t] = G.lower[t];
            a.upper[t] = G.upper[t];
            a.max_step[t] = G.max_step[t];
        }
        a.params = G.params;
        a.crlb = G.crlb;
        a.llr = G.llr;
        a.flags = G.flags;
        a.bad_corners = m.bad_corners;
        const int64_t roi0 = (tile - G.tile0) * m.rois_per_tile;
        const int64_t left = G.n - roi0;
        const int nroi = left < m.rois_per_tile ? (int)left : m.rois_per_tile;
        mixed_dispatch<SCMOS, CLASS>(G.model, G.box, a, roi0, nroi, smem);
        __syncthreads();  // the tile's shared memory is free again
    }
}

// Launch with rois_per_tile (= block size) threads; the class picks the kernel.
cudaError_t launch_mixed_poisson(int cls, const MixedArgs &m, size_t smem, int grid, cudaStream_t s);
cudaError_t launch_mixed_scmos(int cls, const MixedArgs &m, size_t smem, int grid, cudaStream_t s);
int mixed_blocks_per_sm_poisson(int cls, size_t smem);
int mixed_blocks_per_sm_scmos(int cls, size_t smem);
// Set the dynamic shared-memory limit of the family's three kernels on the
// current device (a per-device set-up step of the no-allocation entry point).
cudaError_t mixed_set_attributes_poisson();
cudaError_t mixed_set_attributes_scmos();

inline cudaError_t launch_mixed(bool scmos, int cls, const MixedArgs &m, size_t smem, int grid,
                                cudaStream_t s)
{
    return scmos ? launch_mixed_scmos(cls, m, smem, grid, s)
                 : launch_mixed_poisson(cls, m, smem, grid, s);
}
inline int mixed_blocks_per_sm(bool scmos, int cls, size_t smem)
{
    return scmos ? mixed_blocks_per_sm_scmos(cls, smem) : mixed_blocks_per_sm_poisson(cls, smem);
}

// Dynamic shared memory the mixed kernel may request: well under the 227 KiB
// per-block limit, which also has to hold the kernel's static tile index (a
// 15x15 sCMOS tile of 32 ROIs needs about 58 KiB).
constexpr int kMixedMaxSmem = 200 * 1024;

}  // namespace gmle
