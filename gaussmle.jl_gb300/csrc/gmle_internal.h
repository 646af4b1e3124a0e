// gmle_internal.h - host-side internals shared by the runtime translation units
// (context, pipeline slots, mixed-batch buffers, serving loop, error helpers).
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

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

// Group table of one mixed-batch launch: header {groups, tiles} and group
// descriptors, built in pinned host memory and copied to the device before
// the launch (one copy of 64 + 192 * groups bytes); and the device
// work-stealing tile counter.
constexpr size_t kTableHeader = 64;
struct MixedBufs {
    char *h_base = nullptr, *d_base = nullptr;
    gmle::GroupDesc *h_groups = nullptr, *d_groups = nullptr;
    int64_t *h_header = nullptr, *d_header = nullptr;
    unsigned long long *d_counter = nullptr;
    int cap = 0;
    cudaEvent_t reuse = nullptr;  // the last H2D of this table has completed
};

// Shared-memory classes of the mixed kernel: ROIs up to 9x9, 11x11, 13x13 and
// up.  Each class present gets its own persistent launch, sized for its
// largest box, so that small ROIs keep their occupancy.
constexpr int kClasses = 3;
using gmle::box_class;
using gmle::class_tile;

// Group tables, fork streams and events of one mixed-batch submitter (the
// context's synchronous path, or one slot of the serving loop).
struct MixedSet {
    MixedBufs bufs[2][kClasses];  // [camera family][class]
    // The kernels read the tables from pinned host memory (no copy).  The
    // serving loop does so: a table copy would queue on the copy engine
    // behind the inputs of every admitted request.
    bool zero_copy = false;
    cudaStream_t fork[kClasses] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kClasses] = {};
};

// What one mixed submission launches: per (family, class), tiles, shared
// memory and grid; the graph key of the serving loop is the smem vector.
struct MixedPlan {
    int64_t tiles[2][kClasses] = {};
    size_t smem[2][kClasses] = {};
    int grid[2][kClasses] = {};
    std::vector<gmle_group> plain;  // groups fitted by their own plain launch
};

// Groups of at least this many ROIs fill the GPU on their own: a batch
// submission gives them their (autotuned) plain launch instead of the
// persistent kernel; the serving loop keeps every request in the persistent
// launches, whose captured graphs must not depend on request pointers.
constexpr int64_t kPlainGroupRois = 65536;

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
    gmle_rt::MixedSet mixed;      // the synchronous mixed-batch submitter
    gmle_rt::Server *server = nullptr;
};

namespace gmle_rt {

gmle_status fail(gmle_ctx *ctx, gmle_status st, const char *fmt, ...);
gmle_status cuda_fail(gmle_ctx *ctx, cudaError_t e, const char *what);
gmle_status check_desc(gmle_ctx *ctx, const gmle_fit_desc *d);
int nparams(int model);

gmle_status init_mixed_set(gmle_ctx *ctx, MixedSet &m);
void free_mixed_set(MixedSet &m);
// Validate the groups and fill the pinned tables of every (family, class);
// with allow_plain, groups of kPlainGroupRois or more go to plan.plain.
gmle_status plan_mixed(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups, MixedSet &m,
                       MixedPlan &plan, bool allow_plain);
// Copy the plan's tables to the device on s (not part of a captured graph);
// with record_reuse each table's reuse event is recorded after its copy.
gmle_status upload_plan(gmle_ctx *ctx, MixedSet &m, const MixedPlan &plan, cudaStream_t s,
                        bool record_reuse);
// The plan's plain launches on s, then one persistent launch per (family,
// class), the classes concurrently on m.fork, joined back into s.
gmle_status enqueue_plan(gmle_ctx *ctx, MixedSet &m, const MixedPlan &plan, cudaStream_t s);
gmle_status validate_groups(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups);
gmle_status ensure_mixed(gmle_ctx *ctx, MixedBufs &b, int ngroups);
// Fill b's pinned table for one camera family, with tiles of `tile` ROIs;
// returns its number of tiles.
int64_t build_mixed_table(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups, bool scmos,
                          int tile, MixedBufs &b, gmle_status *st);
// Counter reset and kernel launch of class `cls` over the table in b (the
// caller records b.reuse, or keeps b untouched until the launch has finished).
gmle_status enqueue_mixed(gmle_ctx *ctx, bool scmos, int cls, MixedBufs &b, size_t smem, int grid,
                          cudaStream_t s, bool zero_copy);
int mixed_grid(gmle_ctx *ctx, bool scmos, int cls, size_t smem);
gmle_status free_mixed(MixedBufs &b);
size_t mixed_smem(const gmle_group *groups, int32_t ngroups, bool scmos, int tile);

void server_destroy(gmle_ctx *ctx);

}  // namespace gmle_rt

#define GMLE_CK(call, what)                                                    \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) return gmle_rt::cuda_fail(ctx, e_, what);       \
    } while (0)
