// gmle_frames.cu - ROI extraction from device-resident camera frames.
//
// In the reference pipeline a box finder cuts box x box ROIs out of the image
// stack on the host and hands GaussMLE a ROIBatch of (ROI stack, corners,
// frame indices) (examples/full_pipeline_boxer.jl:72-103; the box finder,
// SMLMBoxer.getboxes, is an external package).  With the frames already on the
// GPU, gmle_cut_rois_device builds the same (box, box, n) stack there, so no
// ROI data crosses the host link.
//
// Layouts (Julia's): frames are Float32 (ny, nx, nframes) column-major, pixel
// (row y, column x, frame f) at (y-1) + ny (x-1) + ny nx (f-1); corners and
// frame indices are 1-based Int32; ROI pixel (i, j) of ROI k is frame pixel
// (y_k + i - 1, x_k + j - 1, f_k), stored at (i-1) + box (j-1) + box^2 k.
//
// The copy is bound by HBM bandwidth: per ROI box^2 * 4 bytes are read and
// written, plus 12 bytes of coordinates.  Each block takes whole ROIs; its
// consecutive threads write consecutive output pixels (coalesced stores), and
// a run of `box` threads reads one ROI column, contiguous in the frame.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "gmle_internal.h"

namespace {

constexpr int kCutThreads = 256;
constexpr int kCutPixels = 2048;  // output pixels per block (whole ROIs)
static_assert(kCutPixels % kCutThreads == 0, "whole pixels per thread");

__global__ void __launch_bounds__(kCutThreads)
    cut_rois_kernel(const float *__restrict__ frames, int32_t ny, int32_t nx, int64_t nframes,
                    const int32_t *__restrict__ fidx, const int32_t *__restrict__ xc,
                    const int32_t *__restrict__ yc, int64_t n, int box, int rois_per_block,
                    float *__restrict__ out, unsigned long long *bad)
{
    __shared__ long long s_base[kCutPixels];  // frame offset of each ROI's first pixel, -1: bad
    const int64_t k0 = (int64_t)blockIdx.x * rois_per_block;
    const int64_t left = n - k0;
    const int nk = left < rois_per_block ? (int)left : rois_per_block;
    if (nk <= 0) return;
    for (int q = threadIdx.x; q < nk; q += blockDim.x) {
        const int64_t k = k0 + q;
        const int32_t f = fidx[k], x0 = xc[k], y0 = yc[k];
        const bool ok = f >= 1 && f <= nframes && x0 >= 1 && y0 >= 1 &&
                        (int64_t)x0 + box - 1 <= nx && (int64_t)y0 + box - 1 <= ny;
        s_base[q] = ok ? (long long)(f - 1) * ny * nx + (long long)(x0 - 1) * ny + (y0 - 1) : -1;
        if (!ok) atomicAdd(bad, 1ull);
    }
    __syncthreads();
    const int b2 = box * box;
    const int cnt = nk * b2;
    float *dst = out + k0 * b2;
    const float qnan = __int_as_float(0x7fc00000);
    // all of a thread's gathers are issued before its first store, so that
    // kCutPixels / kCutThreads loads per thread are in flight at once
    constexpr int U = kCutPixels / kCutThreads;
    float v[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int e = threadIdx.x + u * kCutThreads;
        v[u] = qnan;
        if (e < cnt) {
            const int q = e / b2;
            const int p = e - q * b2;
            const int j = p / box, i = p - j * box;
            const long long base = s_base[q];
            if (base >= 0) v[u] = __ldg(frames + base + (long long)j * ny + i);
        }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
        const int e = threadIdx.x + u * kCutThreads;
        if (e < cnt) dst[e] = v[u];
    }
}

}  // namespace

extern "C" gmle_status gmle_cut_rois_device(gmle_ctx *ctx, const float *d_frames, int32_t ny,
                                            int32_t nx, int64_t nframes,
                                            const int32_t *d_frame_idx,
                                            const int32_t *d_x_corners,
                                            const int32_t *d_y_corners, int64_t n, int32_t box,
                                            float *d_rois, void *stream)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (n < 0) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "n < 0");
    if (n == 0) return GMLE_OK;
    if (box < 1 || box > 32)
        return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "box %d outside 1..32", box);
    if (ny < box || nx < box || nframes < 1)
        return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "frames of %d x %d x %lld cannot hold a %d box",
                             ny, nx, (long long)nframes, box);
    if (!d_frames || !d_frame_idx || !d_x_corners || !d_y_corners || !d_rois)
        return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "frames, frame indices, corners and output "
                                                    "are required");
    cudaSetDevice(ctx->device);
    const int rpb = std::max(1, kCutPixels / (box * box));
    const int64_t blocks = (n + rpb - 1) / rpb;
    if (blocks > 0x7fffffffLL) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "too many ROIs");
    ctx->launches++;
    cut_rois_kernel<<<(unsigned)blocks, kCutThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        d_frames, ny, nx, nframes, d_frame_idx, d_x_corners, d_y_corners, n, box, rpb, d_rois,
        ctx->d_bad);
    GMLE_CK(cudaGetLastError(), "ROI cut kernel launch");
    return GMLE_OK;
}
