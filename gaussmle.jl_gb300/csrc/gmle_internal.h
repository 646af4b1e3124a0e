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
#include "gmle_generic.h"
#include "gmle_launch.cuh"

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

// Launch kinds of a mixed batch: one table launch per (camera family, PSF
// model, box size) present.
constexpr int kKinds = 2 * 4 * gmle::kNumBoxes;
inline int kind_of(const gmle_fit_desc &d)
{
    return ((d.camera != GMLE_CAMERA_POISSON) * 4 + d.model) * gmle::kNumBoxes +
           gmle::box_index(d.box);
}

// Group table of one table launch (gmle::TileTable), built in pinned host
// memory at fixed offsets:
//   [0, 64)              header {groups, tiles}
//   [64, +cap_groups)    per group its KernelArgs
//   [tiles_off, +cap_tiles)  per tile (group << 32) | local tile
// The kernels read it in place (zero copy) or from its device copy.
constexpr size_t kTableHeader = 64;
struct TableBufs {
    char *h_base = nullptr, *d_base = nullptr;
    bool in_pool = false;  // h_base points into the set's pool (not freed on its own)
    int64_t cap_groups = 0, cap_tiles = 0;
    unsigned long long *d_counter = nullptr;
    cudaEvent_t reuse = nullptr;  // the last copy reading h_base has completed
    cudaEvent_t used = nullptr;   // the last launch reading d_base has completed
    size_t tiles_off() const
    {
        return kTableHeader + sizeof(gmle::KernelArgs) * (size_t)cap_groups;
    }
    size_t bytes() const { return tiles_off() + sizeof(int64_t) * (size_t)cap_tiles; }
};

// Group tables, fork streams and events of one mixed-batch submitter (the
// context's synchronous path, or one slot of the serving loop).
constexpr int kForks = 4;
struct MixedSet {
    TableBufs tables[kKinds];
    // The kernels read the tables from pinned host memory (no copy).  The
    // serving loop does so: a table copy would queue on the copy engine
    // behind the inputs of every admitted request.
    bool zero_copy = false;
    // Optional pinned pool (zero-copy sets with one-block-per-tile launches):
    // each plan carves every kind's table out of it from the start, so a plan
    // allocates nothing.  The set must not be planned again before its last
    // plan's launches end.
    char *pool = nullptr;
    size_t pool_bytes = 0, pool_used = 0;
    cudaStream_t fork[kForks] = {};
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join[kForks] = {};
};

// One table launch of a plan.
struct TableLaunch {
    int kind = -1, model = 0, box = 0;
    bool scmos = false;
    bool persistent = true;  // false: one block per tile (no tile counter)
    gmle::LaunchShape shape{};
    int64_t groups = 0, tiles = 0;
};

// What one mixed submission launches: plain launches of large groups, then
// one table launch per kind present.
struct MixedPlan {
    std::vector<TableLaunch> launches;
    std::vector<gmle_group> plain;  // groups fitted by their own plain launch
};

// Groups of at least this many ROIs fill the GPU on their own: a batch
// submission gives them their (autotuned) plain launch instead of a table
// launch; the serving loop keeps every request in the table launches, whose
// captured graphs must not depend on request pointers.
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
    float *d_pv = nullptr;        // gmle_pvalues: device llr and p-values
    int64_t pv_cap = 0;
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
// How a table launch picks its shape: from the context's tuning for the
// kind, else the size-based default for `shape_rois` ROIs (0: the kind's ROIs
// in this submission).  Persistent grids are full (SMs x resident blocks)
// when `full_grid`, else no larger than the tiles.
struct PlanOptions {
    bool allow_plain = true;
    int64_t shape_rois = 0;
    // persistent table launches (a grid of resident blocks that take tiles from
    // a counter; full_grid: sized for the GPU whatever the tiles) or one block
    // per tile
    bool persistent = true;
    bool full_grid = false;
    // table capacity to reserve: groups, and tiles for this many ROIs
    int64_t reserve_groups = 0, reserve_rois = 0;
};
// Validate the groups and fill the pinned tables of every kind present.
gmle_status plan_mixed(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups, MixedSet &m,
                       MixedPlan &plan, const PlanOptions &opt);
// Copy the plan's tables to the device on s (not for zero-copy sets); with
// record_reuse each table's reuse event is recorded after its copy.
gmle_status upload_plan(gmle_ctx *ctx, MixedSet &m, const MixedPlan &plan, cudaStream_t s,
                        bool record_reuse);
// Whether a launch's kernel keeps tensor memory for its whole duration (the
// one-thread-per-ROI sCMOS kernel, which holds its variance tiles there).
inline bool holds_tmem(bool scmos, int tpr) { return scmos && tpr == 1; }
// Fork stream of a plan's index-th launch among nf forks.
int plan_stream(int index, bool holds_tmem, int nf);
// One table launch of a plan on q: its tile counter reset, then the kernel.
gmle_status enqueue_table_launch(gmle_ctx *ctx, MixedSet &m, const TableLaunch &L, cudaStream_t q);
// The plan's plain launches on s, then its table launches, concurrently on
// m.fork when there are several, joined back into s.
gmle_status enqueue_plan(gmle_ctx *ctx, MixedSet &m, const MixedPlan &plan, cudaStream_t s);
gmle_status validate_groups(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups);
Tuning pick_tuning(gmle_ctx *ctx, const gmle_fit_desc *d, int64_t n);
Tuning default_tuning(int num_sms, int model, int box, bool scmos, int64_t n);
gmle::KernelArgs make_args(gmle_ctx *ctx, const gmle_fit_desc *d, const float *data,
                           const int32_t *xc, const int32_t *yc, int64_t n, float *params,
                           float *crlb, float *llr, uint8_t *flags, int tpr);

void server_destroy(gmle_ctx *ctx);

}  // namespace gmle_rt

#define GMLE_CK(call, what)                                                    \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) return gmle_rt::cuda_fail(ctx, e_, what);       \
    } while (0)
