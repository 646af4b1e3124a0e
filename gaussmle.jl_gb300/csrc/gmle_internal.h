// gmle_internal.h - host-side internals shared by the runtime translation units
// (context, pipeline slots, mixed-batch buffers, serving loop, error helpers).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "../../include/gaussmle_gb300.h"
#include "gmle_launch.cuh"
#include "gmle_mixed.cuh"

namespace gmle_rt {

struct Tuning {
    int tpr;
    int rois_per_block;
};

// One pipeline slot of device buffers for the host-buffer path.
struct Slot {
    float *data = nullptr;
    int32_t *xc = nullptr, *yc = nullptr;
    float *params = nullptr, *crlb = nullptr, *llr = nullptr;
    uint8_t *flags = nullptr;
    int64_t cap_rois = 0;   // ROIs the buffers hold
    int64_t cap_b2 = 0;     // box^2 the data buffer was sized for
    // pinned staging for pageable caller memory
    float *h_data = nullptr;
    float *h_params = nullptr, *h_crlb = nullptr, *h_llr = nullptr;
    uint8_t *h_flags = nullptr;
    int64_t h_cap_rois = 0, h_cap_b2 = 0;
    cudaEvent_t h2d_done = nullptr, fit_done = nullptr, d2h_done = nullptr;
    // pending copy of pinned outputs to pageable caller memory
    bool pending = false;
    float *dst_params = nullptr, *dst_crlb = nullptr, *dst_llr = nullptr;
    uint8_t *dst_flags = nullptr;
    int64_t pend_rois = 0;
    int pend_p = 0;
};

// Group table of one mixed-batch launch, in pinned host memory that the
// kernel reads directly, its header {groups, tiles}, and the device
// work-stealing tile counter.
struct MixedBufs {
    gmle::GroupDesc *h_groups = nullptr;
    int64_t *h_header = nullptr;
    unsigned long long *d_counter = nullptr;
    int cap = 0;
    cudaEvent_t reuse = nullptr;  // the last H2D of this table has completed
};

struct Server;

}  // namespace gmle_rt

struct gmle_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t s_fit = nullptr, s_h2d = nullptr, s_d2h = nullptr;
    std::string err;
    std::mutex mu;
    // resident calibration maps, (ny, nx) column-major
    float *d_var = nullptr, *d_gain = nullptr, *d_offset = nullptr;
    int32_t ny = 0, nx = 0;
    unsigned long long *d_bad = nullptr;
    int64_t launches = 0;
    std::map<std::tuple<int, int, int>, gmle_rt::Tuning> tuning;
    gmle_rt::Slot slots[2];
    gmle_rt::MixedBufs mixed[2];  // one group table per camera family
    gmle_rt::Server *server = nullptr;
};

namespace gmle_rt {

gmle_status fail(gmle_ctx *ctx, gmle_status st, const char *fmt, ...);
gmle_status cuda_fail(gmle_ctx *ctx, cudaError_t e, const char *what);
gmle_status check_desc(gmle_ctx *ctx, const gmle_fit_desc *d);
int nparams(int model);

// Launch the persistent mixed-batch kernel(s) for groups of device-resident
// ROIs on stream s, using the table buffers `bufs` (one per camera family).
gmle_status run_mixed(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups, cudaStream_t s,
                      MixedBufs *bufs);
gmle_status validate_groups(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups);
gmle_status ensure_mixed(gmle_ctx *ctx, MixedBufs &b, int ngroups);
// Fill b's pinned table for one camera family; returns its number of tiles.
int64_t build_mixed_table(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups, bool scmos,
                          MixedBufs &b, gmle_status *st);
// Counter reset and kernel launch over the table in b (the caller records
// b.reuse, or otherwise keeps b untouched until the launch has finished).
gmle_status enqueue_mixed(gmle_ctx *ctx, bool scmos, MixedBufs &b, size_t smem, int grid,
                          cudaStream_t s);
int mixed_grid(gmle_ctx *ctx, bool scmos, size_t smem);
gmle_status free_mixed(MixedBufs &b);
size_t mixed_smem(const gmle_group *groups, int32_t ngroups, bool scmos);

void server_destroy(gmle_ctx *ctx);

}  // namespace gmle_rt

#define GMLE_CK(call, what)                                                    \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) return gmle_rt::cuda_fail(ctx, e_, what);       \
    } while (0)
