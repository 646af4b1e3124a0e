// gmle_launch.cuh - launch of one fit-kernel specialisation.
//
// The kernels of one PSF model and camera family are compiled in three parts,
// each its own translation unit (gmle_fit_family.cu, compiled once per
// (model, camera family, part) with -D defines, so the 24 units compile in
// parallel):
//   part 0  one thread per ROI (fit_kernel_r1), odd boxes 5..15;
//   part 1  one thread per ROI, boxes 3, 4, 6, 8, 10, 12, 14, 16;
//   part 2  several lanes per ROI (fit_kernel): 2, 4 and 8 lanes for odd
//           boxes 5..15, 4 lanes for the others.
// Other translation units see the parts through extern template declarations.
#pragma once

#include <algorithm>

#include "gmle_fit_kernel.cuh"

namespace gmle {

// Box sizes with a compiled specialisation: every edge length 3..16 (the
// configurations use 7..15; the reference accepts any box >= 3,
// src/interface.jl:22).  Larger boxes run in the runtime-box kernel
// (gmle_fit_generic.cu).
constexpr int kMinBox = 3, kMaxBox = 16;
constexpr int kNumBoxes = kMaxBox - kMinBox + 1;

__host__ __device__ constexpr int box_index(int box)
{
    return box >= kMinBox && box <= kMaxBox ? box - kMinBox : -1;
}
__host__ __device__ constexpr int box_of_index(int k) { return k + kMinBox; }

inline bool box_supported(int box) { return box_index(box) >= 0; }

// The part of the odd boxes 5..15 (the most used sizes, with 8-lane kernels).
__host__ __device__ constexpr bool main_box(int box) { return box >= 5 && box <= 15 && (box & 1); }

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

// Lanes per ROI with a compiled kernel: 1 (fit_kernel_r1) for every box; 4
// (fit_kernel) for every box; 2 and 8 for the odd boxes 5..15.
inline bool tpr_supported(int tpr, int box)
{
    return tpr == 1 || tpr == 4 || ((tpr == 2 || tpr == 8) && main_box(box));
}

// Part holding the kernel of a launch shape (see the top of this file).
__host__ __device__ constexpr int part_of(int box, int tpr) { return tpr == 1 ? (main_box(box) ? 0 : 1) : 2; }

template <int MODEL, bool SCMOS, int PART>
cudaError_t launch_part(int box, const KernelArgs &a, const TileTable &t, const LaunchShape &shape,
                        cudaStream_t s);
template <int MODEL, bool SCMOS, int PART>
int table_blocks_part(int box, int tpr, int rois_per_block);

inline cudaError_t launch_fit(int model, int box, bool scmos, const KernelArgs &a,
                              const TileTable &t, const LaunchShape &shape, cudaStream_t s)
{
    if (!box_supported(box) || !tpr_supported(shape.tpr, box)) return cudaErrorInvalidValue;
    const int part = part_of(box, shape.tpr);
#define GMLE_CASE(M)                                                                       \
    case M:                                                                                \
        if (part == 0)                                                                     \
            return scmos ? launch_part<M, true, 0>(box, a, t, shape, s)                    \
                         : launch_part<M, false, 0>(box, a, t, shape, s);                  \
        if (part == 1)                                                                     \
            return scmos ? launch_part<M, true, 1>(box, a, t, shape, s)                    \
                         : launch_part<M, false, 1>(box, a, t, shape, s);                  \
        return scmos ? launch_part<M, true, 2>(box, a, t, shape, s)                        \
                     : launch_part<M, false, 2>(box, a, t, shape, s);
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
    if (!box_supported(box) || !tpr_supported(tpr, box)) return -(int)cudaErrorInvalidValue;
    const int part = part_of(box, tpr);
#define GMLE_CASE(M)                                                                       \
    case M:                                                                                \
        if (part == 0)                                                                     \
            return scmos ? table_blocks_part<M, true, 0>(box, tpr, rois_per_block)         \
                         : table_blocks_part<M, false, 0>(box, tpr, rois_per_block);       \
        if (part == 1)                                                                     \
            return scmos ? table_blocks_part<M, true, 1>(box, tpr, rois_per_block)         \
                         : table_blocks_part<M, false, 1>(box, tpr, rois_per_block);       \
        return scmos ? table_blocks_part<M, true, 2>(box, tpr, rois_per_block)             \
                     : table_blocks_part<M, false, 2>(box, tpr, rois_per_block);
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

// The kernels of a part.  PART is a template parameter (not the GMLE_PART
// macro of the unit that compiles them) so that the instantiations of two
// parts never share a name: template instantiations of the same name are
// merged at link time.  They are instantiated in gmle_fit_family.cu only.
template <int MODEL, int BOX, bool SCMOS, int PART>
cudaError_t kernel_for(int tpr, bool table, bool lm, FitKernel *kern)
{
    constexpr int R1PART = part_of(BOX, 1);  // this box's one-thread part
    const bool r1 = tpr == 1;
    if (lm && (!r1 || table)) return cudaErrorInvalidConfiguration;
    if (!tpr_supported(tpr, BOX)) return cudaErrorInvalidConfiguration;
    if constexpr (PART == R1PART) {
        if (!r1) return cudaErrorInvalidConfiguration;
        if (lm) *kern = fit_kernel_r1<MODEL, BOX, SCMOS, false, true>;
        else *kern = table ? fit_kernel_r1<MODEL, BOX, SCMOS, true> : fit_kernel_r1<MODEL, BOX, SCMOS, false>;
    } else if constexpr (PART == 2) {
        if (r1) return cudaErrorInvalidConfiguration;
        if (tpr == 4) {
            *kern = table ? fit_kernel<MODEL, BOX, SCMOS, true, 4> : fit_kernel<MODEL, BOX, SCMOS, false, 4>;
        } else if constexpr (main_box(BOX)) {
            if (tpr == 2)
                *kern = table ? fit_kernel<MODEL, BOX, SCMOS, true, 2> : fit_kernel<MODEL, BOX, SCMOS, false, 2>;
            else
                *kern = table ? fit_kernel<MODEL, BOX, SCMOS, true, 8> : fit_kernel<MODEL, BOX, SCMOS, false, 8>;
        }
    } else {
        return cudaErrorInvalidConfiguration;
    }
    // The largest dynamic shared memory a block may have, once per kernel and
    // device (setting it twice is harmless).
    constexpr int kMaxDevices = 64;
    static bool done[2][4][2][kMaxDevices] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const bool known = dev >= 0 && dev < kMaxDevices;
    const int ti = tpr == 1 ? 0 : tpr == 2 ? 1 : tpr == 4 ? 2 : 3;
    if (known && done[lm][ti][table][dev]) return cudaSuccess;
    // the 227 KiB a block may use include the kernel's static shared memory
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, *kern);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(*kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             227 * 1024 - (int)fa.sharedSizeBytes);
    if (e == cudaSuccess && known) done[lm][ti][table][dev] = true;
    return e;
}

template <int MODEL, int BOX, bool SCMOS, int PART>
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
    cudaError_t e = kernel_for<MODEL, BOX, SCMOS, PART>(tpr, table, shape.lm, &kern);
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

template <int MODEL, int BOX, bool SCMOS, int PART>
int table_blocks_one(int tpr, int rpb)
{
    FitKernel kern;
    cudaError_t e = kernel_for<MODEL, BOX, SCMOS, PART>(tpr, true, false, &kern);
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

#define GMLE_CASE_PART0(CALL) CALL(5) CALL(7) CALL(9) CALL(11) CALL(13) CALL(15)
#define GMLE_CASE_PART1(CALL) CALL(3) CALL(4) CALL(6) CALL(8) CALL(10) CALL(12) CALL(14) CALL(16)
#define GMLE_CASE_PART2(CALL) GMLE_CASE_PART0(CALL) GMLE_CASE_PART1(CALL)

// A part's boxes: odd 5..15 (part 0), the other boxes 3..16 (part 1), all
// boxes 3..16 (part 2).
#define GMLE_PART_SWITCH(GMLE_CASE)                                 \
    if constexpr (PART == 0) {                                      \
        switch (box) { GMLE_CASE_PART0(GMLE_CASE) default: break; } \
    } else if constexpr (PART == 1) {                               \
        switch (box) { GMLE_CASE_PART1(GMLE_CASE) default: break; } \
    } else {                                                        \
        switch (box) { GMLE_CASE_PART2(GMLE_CASE) default: break; } \
    }

template <int MODEL, bool SCMOS, int PART>
cudaError_t launch_part(int box, const KernelArgs &a, const TileTable &t, const LaunchShape &shape,
                        cudaStream_t s)
{
#define GMLE_CASE(B) case B: return launch_one<MODEL, B, SCMOS, PART>(a, t, shape, s);
    GMLE_PART_SWITCH(GMLE_CASE)
#undef GMLE_CASE
    return cudaErrorInvalidValue;
}

template <int MODEL, bool SCMOS, int PART>
int table_blocks_part(int box, int tpr, int rpb)
{
#define GMLE_CASE(B) case B: return table_blocks_one<MODEL, B, SCMOS, PART>(tpr, rpb);
    GMLE_PART_SWITCH(GMLE_CASE)
#undef GMLE_CASE
    return 0;
}
#undef GMLE_PART_SWITCH

#define GMLE_EXTERN_PART(M, S, P)                                                            \
    extern template cudaError_t launch_part<M, S, P>(int, const KernelArgs &, const TileTable &, \
                                                     const LaunchShape &, cudaStream_t);      \
    extern template int table_blocks_part<M, S, P>(int, int, int);
#define GMLE_EXTERN_MODEL(M)                                                         \
    GMLE_EXTERN_PART(M, false, 0) GMLE_EXTERN_PART(M, false, 1) GMLE_EXTERN_PART(M, false, 2) \
    GMLE_EXTERN_PART(M, true, 0) GMLE_EXTERN_PART(M, true, 1) GMLE_EXTERN_PART(M, true, 2)
GMLE_EXTERN_MODEL(0) GMLE_EXTERN_MODEL(1) GMLE_EXTERN_MODEL(2) GMLE_EXTERN_MODEL(3)
#undef GMLE_EXTERN_MODEL
#undef GMLE_EXTERN_PART

}  // namespace gmle
