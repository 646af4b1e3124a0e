// gmle_launch.cuh - launch of one fit-kernel specialisation.  Each
// gmle_fit_<model>_<camera family>.cu translation unit instantiates the
// kernels of one PSF model and camera family for every supported box size, so
// the eight units compile in parallel.
#pragma once

#include <algorithm>

#include "gmle_fit_kernel.cuh"

namespace gmle {

// Box sizes with a compiled specialisation (the configurations use 7..15).
constexpr int kBoxes[] = {5, 7, 9, 11, 13, 15};
constexpr int kNumBoxes = 6;

__host__ __device__ constexpr int box_index(int box)
{
    return box == 5 ? 0 : box == 7 ? 1 : box == 9 ? 2 : box == 11 ? 3 : box == 13 ? 4
                                                                     : box == 15 ? 5 : -1;
}

inline bool box_supported(int box) { return box_index(box) >= 0; }

// Largest block of the one-thread-per-ROI kernel (its __launch_bounds__).
constexpr int kMaxThreadsR1 = 128;

// One launch of a model's kernel.  Plain (t.header == nullptr): ceil(a.n / rpb)
// blocks over `a`.  Table: `grid` persistent blocks over the table's groups,
// whose arguments carry this launch's tpr; `a` then only supplies tpr.  `lm`
// selects the full-Hessian method, which runs in plain one-thread-per-ROI
// launches only.
struct LaunchShape {
    int tpr;
    int rois_per_block;
    int64_t grid;  // table launches only
    bool lm = false;
};

#define GMLE_DECLARE_FAMILY(M, FAM)                                                           \
    cudaError_t launch_fit_m##M##_##FAM(int box, const KernelArgs &a, const TileTable &t,     \
                                        const LaunchShape &shape, cudaStream_t s);            \
    int table_blocks_m##M##_##FAM(int box, int tpr, int rois_per_block);
GMLE_DECLARE_FAMILY(0, poisson) GMLE_DECLARE_FAMILY(0, scmos)
GMLE_DECLARE_FAMILY(1, poisson) GMLE_DECLARE_FAMILY(1, scmos)
GMLE_DECLARE_FAMILY(2, poisson) GMLE_DECLARE_FAMILY(2, scmos)
GMLE_DECLARE_FAMILY(3, poisson) GMLE_DECLARE_FAMILY(3, scmos)
#undef GMLE_DECLARE_FAMILY

inline cudaError_t launch_fit(int model, int box, bool scmos, const KernelArgs &a,
                              const TileTable &t, const LaunchShape &shape, cudaStream_t s)
{
#define GMLE_CASE(M)                                                        \
    case M:                                                                 \
        return scmos ? launch_fit_m##M##_scmos(box, a, t, shape, s)         \
                     : launch_fit_m##M##_poisson(box, a, t, shape, s);
    switch (model) {
        GMLE_CASE(0) GMLE_CASE(1) GMLE_CASE(2) GMLE_CASE(3)
        default: return cudaErrorInvalidValue;
    }
#undef GMLE_CASE
}

// Resident blocks per SM of a table launch of this shape (0 if none fits; a
// negated cudaError_t on error); also sets the kernel's shared-memory limit on
// the current device.
inline int table_blocks_per_sm(int model, int box, bool scmos, int tpr, int rois_per_block)
{
#define GMLE_CASE(M)                                                        \
    case M:                                                                 \
        return scmos ? table_blocks_m##M##_scmos(box, tpr, rois_per_block)  \
                     : table_blocks_m##M##_poisson(box, tpr, rois_per_block);
    switch (model) {
        GMLE_CASE(0) GMLE_CASE(1) GMLE_CASE(2) GMLE_CASE(3)
        default: return 0;
    }
#undef GMLE_CASE
}

// Dynamic shared memory of a launch (table launches add the block's slot).
inline size_t launch_smem(int model, int box, bool scmos, int tpr, int rpb, bool table)
{
    const size_t s = smem_bytes(model, box, scmos, tpr, rpb);
    return table ? table_smem_bytes(s) : s;
}

using FitKernel = void (*)(const KernelArgs, const TileTable);

template <int MODEL, int BOX, bool SCMOS>
cudaError_t kernel_for(int tpr, bool table, bool lm, FitKernel *kern)
{
    const bool r1 = tpr == 1;
    if (lm && (!r1 || table)) return cudaErrorInvalidConfiguration;
    *kern = lm ? fit_kernel_r1<MODEL, BOX, SCMOS, false, true>
          : r1 ? (table ? fit_kernel_r1<MODEL, BOX, SCMOS, true> : fit_kernel_r1<MODEL, BOX, SCMOS, false>)
               : (table ? fit_kernel<MODEL, BOX, SCMOS, true> : fit_kernel<MODEL, BOX, SCMOS, false>);
    // The largest dynamic shared memory a block may have, once per kernel and
    // device (setting it twice is harmless).
    constexpr int kMaxDevices = 64;
    static bool done[2][2][2][kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const bool known = dev >= 0 && dev < kMaxDevices;
    if (known && done[lm][r1][table][dev]) return cudaSuccess;
    // the 227 KiB a block may use include the kernel's static shared memory
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, *kern);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(*kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024 - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess && known) done[lm][r1][table][dev] = true;
    return e;
}

template <int MODEL, int BOX, bool SCMOS>
cudaError_t launch_one(const KernelArgs &a, const TileTable &t, const LaunchShape &shape,
                       cudaStream_t s)
{
    const int tpr = shape.tpr, rpb = shape.rois_per_block;
    if (tpr != a.tpr) return cudaErrorInvalidValue;
    const int threads = rpb * tpr;
    const bool table = t.header != nullptr;
    if (tpr == 1 && threads > kMaxThreadsR1) return cudaErrorInvalidConfiguration;
    const size_t smem = launch_smem(MODEL, BOX, SCMOS, tpr, rpb, table);
    FitKernel kern;
    cudaError_t e = kernel_for<MODEL, BOX, SCMOS>(tpr, table, shape.lm, &kern);
    if (e != cudaSuccess) return e;
    const int64_t blocks = table ? shape.grid : (a.n + rpb - 1) / rpb;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    kern<<<(unsigned)blocks, threads, smem, s>>>(a, t);
    return cudaGetLastError();
}

// Resident blocks per SM of a kernel that holds `cols` tensor-memory columns
// per block (a negated cudaError_t on error).
inline int tmem_kernel_blocks_per_sm(FitKernel kern, int threads, size_t dyn_smem, int cols)
{
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kern);
    if (e != cudaSuccess) return -(int)e;
    int dev = 0, regs_sm = 0, smem_sm = 0, smem_rsv = 0, thr_sm = 0, blk_sm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev);
    if (e == cudaSuccess)
        e = cudaDeviceGetAttribute(&blk_sm, cudaDevAttrMaxBlocksPerMultiprocessor, dev);
    if (e != cudaSuccess) return -(int)e;
    const int warps = (threads + 31) / 32;
    const int regs_warp = ((fa.numRegs + 7) / 8) * 8 * 32;  // allocated per warp in 8-register units
    const int by_regs = regs_warp > 0 ? (regs_sm / regs_warp) / warps : blk_sm;
    const size_t per_block = dyn_smem + fa.sharedSizeBytes + (size_t)smem_rsv;
    const int by_smem = (int)((size_t)smem_sm / per_block);
    const int by_threads = thr_sm / (warps * 32);
    const int by_tmem = 512 / cols;
    return std::max(0, std::min({by_regs, by_smem, by_threads, blk_sm, by_tmem}));
}

template <int MODEL, int BOX, bool SCMOS>
int table_blocks_one(int tpr, int rpb)
{
    FitKernel kern;
    cudaError_t e = kernel_for<MODEL, BOX, SCMOS>(tpr, true, false, &kern);
    if (e != cudaSuccess) return -(int)e;
    const size_t smem = launch_smem(MODEL, BOX, SCMOS, tpr, rpb, true);
    int nb = 0;
    if (!(SCMOS && tpr == 1)) {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, rpb * tpr, smem);
        return e == cudaSuccess ? nb : -(int)e;
    }
    // The one-thread sCMOS kernel allocates tensor memory, for which the
    // occupancy API answers one block per SM (it cannot know how many columns
    // a block takes).  Its residency is computed here from its registers,
    // shared memory and threads, and the 512 columns an SM holds.
    return tmem_kernel_blocks_per_sm(kern, rpb * tpr, smem, tmem_var_cols(BOX));
}

#define GMLE_BOX_SWITCH(CALL)       \
    switch (box) {                  \
        case 5: CALL(5)             \
        case 7: CALL(7)             \
        case 9: CALL(9)             \
        case 11: CALL(11)           \
        case 13: CALL(13)           \
        case 15: CALL(15)           \
        default: break;             \
    }

template <int MODEL, bool SCMOS>
cudaError_t launch_family(int box, const KernelArgs &a, const TileTable &t,
                          const LaunchShape &shape, cudaStream_t s)
{
#define GMLE_CASE(B) return launch_one<MODEL, B, SCMOS>(a, t, shape, s);
    GMLE_BOX_SWITCH(GMLE_CASE)
#undef GMLE_CASE
    return cudaErrorInvalidValue;
}

template <int MODEL, bool SCMOS>
int table_blocks_family(int box, int tpr, int rpb)
{
#define GMLE_CASE(B) return table_blocks_one<MODEL, B, SCMOS>(tpr, rpb);
    GMLE_BOX_SWITCH(GMLE_CASE)
#undef GMLE_CASE
    return 0;
}

}  // namespace gmle
