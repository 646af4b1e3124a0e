// gmle_noalloc.cu - gmle_fit_mixed_device_noalloc: the mixed-batch fit for
// callers that cannot allocate device memory.
//
// The persistent mixed-batch kernels (gmle_mixed.cuh) need scratch beyond the
// caller's inputs and outputs: a group table and a header per launch, a
// work-stealing tile counter per launch, and a counter of skipped ROIs.  Here
// that scratch is the file-scope array g_noalloc_scratch, reserved on a device
// when this module is loaded there and held until the process exits:
//
//   [0, 256)    unsigned long long counters[8]: the tile counters of the six
//               (camera family, shared-memory class) launches, then the
//               skipped-ROI counter.  A tile counter must be zero when its
//               launch starts; every call's table copy writes all of them to
//               zero, on the caller's stream, before its launches.
//   [256, 512)  int64_t headers[6][2]: {groups, tiles} of each launch.
//   [512, ...)  gmle::GroupDesc table[GMLE_NOALLOC_MAX_GROUPS]; each launch
//               reads its own contiguous slice.
//
// A call builds the image of [0, 512 + 192 * groups) in a static host buffer,
// copies it with one cudaMemcpyAsync on the caller's stream (the pageable
// source is consumed before that call returns, so the buffer is reused by the
// next call), then enqueues one persistent launch per (family, class) present
// on the same stream.  It allocates nothing: no cudaMalloc, cudaMallocHost,
// cudaFree, stream or event, and no host heap.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "gmle_internal.h"

namespace {

using gmle::GroupDesc;

constexpr int kMaxGroups = GMLE_NOALLOC_MAX_GROUPS;
constexpr int kLaunches = 2 * gmle_rt::kClasses;  // (camera family, shared-memory class)
constexpr size_t kHeadersOff = 256;
constexpr size_t kTableOff = 512;
constexpr size_t kScratchBytes = kTableOff + sizeof(GroupDesc) * kMaxGroups;
constexpr int kBadCounter = kLaunches;            // index in counters[]
constexpr int kMaxDevices = 64;

static_assert(kScratchBytes == GMLE_NOALLOC_SCRATCH_BYTES, "header and layout disagree");
static_assert(sizeof(unsigned long long) * (kLaunches + 1) <= kHeadersOff, "counters overflow");
static_assert(sizeof(int64_t) * 2 * kLaunches <= kTableOff - kHeadersOff, "headers overflow");
static_assert(sizeof(GroupDesc) % 16 == 0, "table entries keep 16-byte alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Host image of the scratch, and per-device set-up; both under g_mu.
alignas(256) unsigned char g_stage[kScratchBytes];
int g_order[kMaxGroups];
std::mutex g_mu;
struct DeviceState {
    unsigned char *scratch = nullptr;  // cudaGetSymbolAddress of g_noalloc_scratch
    int num_sms = 0;
};
DeviceState g_dev[kMaxDevices];

gmle_status report(char *err, int32_t err_len, gmle_status st, const char *fmt, ...)
{
    if (err && err_len > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)err_len, fmt, ap);
        va_end(ap);
    }
    return st;
}

gmle_status cuda_report(char *err, int32_t err_len, cudaError_t e, const char *what)
{
    return report(err, err_len, e == cudaErrorNoDevice ? GMLE_NO_DEVICE : GMLE_CUDA_ERROR,
                  "%s: %s", what, cudaGetErrorString(e));
}

gmle_status check_group(const gmle_group &G, int k, bool have_var, bool have_adu_maps, char *err,
                        int32_t err_len)
{
    const gmle_fit_desc &d = G.desc;
    if (d.model < 0 || d.model > 3)
        return report(err, err_len, GMLE_UNSUPPORTED_MODEL, "group %d: unknown model id %d", k,
                      d.model);
    if (!gmle::mixed_box(d.box))
        return report(err, err_len, GMLE_UNSUPPORTED_BOX,
                      "group %d: box %d not in the mixed kernel (5..15 odd)", k, d.box);
    if (d.iterations < 0) return report(err, err_len, GMLE_INVALID_ARG, "group %d: iterations < 0", k);
    if (d.camera < 0 || d.camera > 2)
        return report(err, err_len, GMLE_INVALID_ARG, "group %d: unknown camera id %d", k, d.camera);
    if (d.model == GMLE_MODEL_XYNB && !(d.psf[0] > 0.f))
        return report(err, err_len, GMLE_INVALID_ARG, "group %d: GaussianXYNB sigma must be > 0", k);
    if (d.model == GMLE_MODEL_ASTIG && (!(d.psf[0] > 0.f) || !(d.psf[1] > 0.f) || d.psf[7] == 0.f))
        return report(err, err_len, GMLE_INVALID_ARG,
                      "group %d: astigmatic sigma0 must be > 0 and d != 0", k);
    if (G.n < 0) return report(err, err_len, GMLE_INVALID_ARG, "group %d: n < 0", k);
    if (G.n == 0) return GMLE_OK;
    if (!G.data || !G.params || !G.crlb || !G.llr)
        return report(err, err_len, GMLE_INVALID_ARG,
                      "group %d: data and output pointers are required", k);
    if (d.camera != GMLE_CAMERA_POISSON) {
        if (!have_var)
            return report(err, err_len, GMLE_INVALID_ARG,
                          "group %d: sCMOS fit without a variance map", k);
        if (d.camera == GMLE_CAMERA_SCMOS_ADU && !have_adu_maps)
            return report(err, err_len, GMLE_INVALID_ARG,
                          "group %d: ADU fit needs gain and offset maps", k);
        if (!G.x_corners || !G.y_corners)
            return report(err, err_len, GMLE_INVALID_ARG, "group %d: sCMOS fit needs ROI corners",
                          k);
    }
    return GMLE_OK;
}

double group_cost(const gmle_fit_desc &d)
{
    return (double)d.box * d.box * (gmle_rt::nparams(d.model) + (d.model == 3 ? 3 : 0));
}

// First call on the current device: the scratch address and the kernels'
// shared-memory limit.  Called with g_mu held.
gmle_status setup_device(int dev, char *err, int32_t err_len)
{
    DeviceState &S = g_dev[dev];
    if (S.scratch) return GMLE_OK;
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_report(err, err_len, e, "cudaGetSymbolAddress(scratch)");
    int sms = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_report(err, err_len, e, "cudaDeviceGetAttribute");
    e = gmle::mixed_set_attributes_poisson();
    if (e == cudaSuccess) e = gmle::mixed_set_attributes_scmos();
    if (e != cudaSuccess) return cuda_report(err, err_len, e, "cudaFuncSetAttribute(mixed kernels)");
    S.num_sms = sms;
    S.scratch = static_cast<unsigned char *>(p);
    return GMLE_OK;
}

}  // namespace

extern "C" gmle_status gmle_fit_mixed_device_noalloc(const gmle_group *groups, int32_t ngroups,
                                                     const float *variance, const float *gain,
                                                     const float *offset, int32_t ny, int32_t nx,
                                                     void *stream, char *err, int32_t err_len)
{
    if (err && err_len > 0) err[0] = '\0';
    if (ngroups < 0) return report(err, err_len, GMLE_INVALID_ARG, "ngroups < 0");
    if (ngroups > kMaxGroups)
        return report(err, err_len, GMLE_INVALID_ARG,
                      "ngroups %d exceeds the static group table of %d groups "
                      "(GMLE_NOALLOC_MAX_GROUPS); split the batch into several calls",
                      ngroups, kMaxGroups);
    if (ngroups > 0 && !groups) return report(err, err_len, GMLE_INVALID_ARG, "groups is NULL");
    if (variance && (ny <= 0 || nx <= 0))
        return report(err, err_len, GMLE_INVALID_ARG, "calibration maps need ny, nx > 0");
    const bool have_adu_maps = gain && offset;
    for (int k = 0; k < ngroups; k++) {
        gmle_status st = check_group(groups[k], k, variance != nullptr, have_adu_maps, err, err_len);
        if (st != GMLE_OK) return st;
    }

    std::lock_guard<std::mutex> lk(g_mu);
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_report(err, err_len, e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return report(err, err_len, GMLE_INVALID_ARG, "device %d beyond the %d supported", dev,
                      kMaxDevices);
    gmle_status st = setup_device(dev, err, err_len);
    if (st != GMLE_OK) return st;
    const DeviceState &S = g_dev[dev];

    // Host image: zeroed counters, then per launch its header and table slice
    // (groups in decreasing cost, so that the heavy tiles start first).
    std::memset(g_stage, 0, kTableOff);
    unsigned long long *d_counters = reinterpret_cast<unsigned long long *>(S.scratch);
    int64_t *h_headers = reinterpret_cast<int64_t *>(g_stage + kHeadersOff);
    GroupDesc *h_table = reinterpret_cast<GroupDesc *>(g_stage + kTableOff);
    int used = 0;
    int first[kLaunches] = {};
    size_t smem[kLaunches] = {};
    for (int fam = 0; fam < 2; fam++) {
        for (int c = 0; c < gmle_rt::kClasses; c++) {
            const int L = fam * gmle_rt::kClasses + c;
            const int tile = gmle::class_tile(c);
            int cnt = 0;
            for (int k = 0; k < ngroups; k++) {
                const gmle_group &G = groups[k];
                if (G.n > 0 && (G.desc.camera != GMLE_CAMERA_POISSON) == (fam == 1) &&
                    gmle::box_class(G.desc.box) == c)
                    g_order[cnt++] = k;
            }
            first[L] = used;
            if (cnt == 0) continue;
            std::sort(g_order, g_order + cnt, [&](int x, int y) {
                const double cx = group_cost(groups[x].desc), cy = group_cost(groups[y].desc);
                return cx > cy || (cx == cy && x < y);
            });
            int64_t tiles = 0;
            for (int q = 0; q < cnt; q++) {
                const gmle_group &G = groups[g_order[q]];
                GroupDesc &D = h_table[used + q];
                std::memset(&D, 0, sizeof D);
                D.data = G.data;
                D.xc = G.x_corners;
                D.yc = G.y_corners;
                D.n = G.n;
                D.params = G.params;
                D.crlb = G.crlb;
                D.llr = G.llr;
                D.flags = G.flags;
                D.model = G.desc.model;
                D.box = G.desc.box;
                D.iterations = G.desc.iterations;
                D.adu = G.desc.camera == GMLE_CAMERA_SCMOS_ADU;
                std::memcpy(D.psf, G.desc.psf, sizeof D.psf);
                std::memcpy(D.lower, G.desc.lower, sizeof D.lower);
                std::memcpy(D.upper, G.desc.upper, sizeof D.upper);
                std::memcpy(D.max_step, G.desc.max_step, sizeof D.max_step);
                D.tile0 = tiles;
                tiles += (G.n + tile - 1) / tile;
                smem[L] = std::max(smem[L], gmle::smem_bytes(G.desc.model, G.desc.box, fam == 1, 1,
                                                             tile));
            }
            h_headers[2 * L] = cnt;
            h_headers[2 * L + 1] = tiles;
            used += cnt;
        }
    }
    if (used == 0) return GMLE_OK;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    e = cudaMemcpyAsync(S.scratch, g_stage, kTableOff + sizeof(GroupDesc) * (size_t)used,
                        cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) return cuda_report(err, err_len, e, "H2D group tables");
    for (int fam = 0; fam < 2; fam++) {
        for (int c = 0; c < gmle_rt::kClasses; c++) {
            const int L = fam * gmle_rt::kClasses + c;
            if (h_headers[2 * L] == 0) continue;
            const bool scmos = fam == 1;
            gmle::MixedArgs m;
            m.groups = reinterpret_cast<const GroupDesc *>(S.scratch + kTableOff) + first[L];
            m.header = reinterpret_cast<const int64_t *>(S.scratch + kHeadersOff) + 2 * L;
            m.tile_counter = d_counters + L;
            m.var = variance;
            m.gain = gain;
            m.offset = offset;
            m.ny = variance ? ny : 0;
            m.nx = variance ? nx : 0;
            m.rois_per_tile = gmle::class_tile(c);
            m.sqrt2pi = sqrtf(2.0f * (float)3.14159265358979323846);
            m.bad_corners = d_counters + kBadCounter;
            const int grid = S.num_sms * std::max(1, gmle::mixed_blocks_per_sm(scmos, c, smem[L]));
            e = gmle::launch_mixed(scmos, c, m, smem[L], grid, s);
            if (e != cudaSuccess) return cuda_report(err, err_len, e, "mixed kernel launch");
        }
    }
    return GMLE_OK;
}
