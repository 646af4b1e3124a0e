// gmle_noalloc.cu - gmle_fit_mixed_device_noalloc: the mixed-batch fit for
// callers that cannot allocate device memory: hosts whose device memory is held
// by their own pool allocator (CUDA.jl, PyTorch), and code where a cudaMalloc,
// which can synchronise the device, must not happen.
//
// A mixed batch runs as one persistent table launch per (camera family, PSF
// model, box size) present (gmle_fit_kernel.cuh, TileTable).  Those launches
// need scratch beyond the caller's inputs and outputs: per launch a header and
// a work-stealing tile counter, per group its kernel arguments and first
// tile, and a counter of skipped ROIs.  Here that scratch is the file-scope
// array g_noalloc_scratch, reserved on a device when this module is loaded
// there and held until the process exits:
//
//   [0, 1024)      unsigned long long counters[128]: the tile counters of the
//                  112 kinds (2 camera families x 4 models x boxes 3..16),
//                  then the skipped-ROI counter.  A tile counter must be zero
//                  when its launch starts; every call's table write sets all
//                  of them to zero, on the caller's stream, before its
//                  launches.
//   [1024, 3072)   int64_t headers[112][2]: {groups, tiles} of each launch.
//   [3072, 11264)  int64_t tile0[GMLE_NOALLOC_MAX_GROUPS]: each group's first
//                  tile within its launch (the tile's group is found by
//                  binary search, so no per-tile table is needed).
//   [11264, ...)   gmle::KernelArgs args[GMLE_NOALLOC_MAX_GROUPS].
// Each launch reads its own contiguous slice of tile0 and args.
//
// A call builds the image of [0, 11264 + 224 * groups) in a static host buffer,
// then writes it into the scratch with write_scratch launches on the caller's
// stream that carry it in their launch parameters, up to 32 704 bytes each
// (one launch for up to 95 groups, eight for 1024).  Launch parameters are
// copied when a launch is enqueued, so the host buffer is free for the next
// call as soon as this one returns, and nothing waits for the stream: a
// host-to-device copy from the (pageable) buffer could instead make the host
// wait for the stream's earlier work, and would read the buffer again if its
// stream work were replayed.  The fit launches follow on the same stream.  It
// allocates nothing: no cudaMalloc, cudaMallocHost, cudaFree, stream or event,
// and no host heap.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "gmle_internal.h"

namespace {

using gmle::KernelArgs;
using gmle_rt::kKinds;

constexpr int kMaxGroups = GMLE_NOALLOC_MAX_GROUPS;
constexpr size_t kCountersOff = 0;
constexpr int kBadCounter = kKinds;  // index in counters[]
constexpr size_t kHeadersOff = 1024;
constexpr size_t kTile0Off = 3072;
constexpr size_t kArgsOff = kTile0Off + sizeof(int64_t) * kMaxGroups;
constexpr size_t kScratchBytes = kArgsOff + sizeof(KernelArgs) * kMaxGroups;
constexpr int kMaxDevices = 64;

static_assert(kScratchBytes == GMLE_NOALLOC_SCRATCH_BYTES, "header and layout disagree");
static_assert(sizeof(unsigned long long) * (kKinds + 1) <= kHeadersOff, "counters overflow");
static_assert(kHeadersOff + sizeof(int64_t) * 2 * kKinds <= kTile0Off, "headers overflow");
static_assert(sizeof(KernelArgs) % 16 == 0 && kArgsOff % 16 == 0, "16-byte aligned arguments");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// One piece of the host image, carried in a launch's parameters (kernel
// parameters may take up to 32 764 bytes).
constexpr int kChunkBytes = 32704;
struct ScratchChunk {
    uint32_t offset;  // into the scratch, a multiple of 16
    uint32_t bytes;   // a multiple of 16, at most kChunkBytes
    uint32_t pad[2];
    uint4 data[kChunkBytes / 16];
};
static_assert(sizeof(ScratchChunk) <= 32764, "kernel parameter limit");

__global__ void write_scratch(const ScratchChunk c)
{
    uint4 *dst = reinterpret_cast<uint4 *>(g_noalloc_scratch + c.offset);
    for (uint32_t w = threadIdx.x; w < c.bytes / 16; w += blockDim.x) dst[w] = c.data[w];
}

// Host image of the scratch, the launch parameters of its pieces, and
// per-device set-up; all under g_mu.
alignas(256) unsigned char g_stage[kScratchBytes];
ScratchChunk g_chunk;
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
    if (!gmle::box_supported(d.box))
        return report(err, err_len, GMLE_UNSUPPORTED_BOX,
                      "group %d: box size %d: this entry point takes boxes %d..%d", k, d.box,
                      gmle::kMinBox, gmle::kMaxBox);
    if (d.iterations < 0) return report(err, err_len, GMLE_INVALID_ARG, "group %d: iterations < 0", k);
    if (d.camera < 0 || d.camera > 2)
        return report(err, err_len, GMLE_INVALID_ARG, "group %d: unknown camera id %d", k, d.camera);
    if (d.method != GMLE_METHOD_NEWTON)
        return report(err, err_len, GMLE_INVALID_ARG,
                      "group %d: method %d runs through gmle_fit and gmle_fit_device only", k,
                      d.method);
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

// First call on the current device: the scratch address and the SM count.
// Called with g_mu held.
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

    // Host image: zeroed counters, then per kind its header and its slice of
    // the group arguments and first tiles.
    std::memset(g_stage, 0, kTile0Off);
    int64_t *h_headers = reinterpret_cast<int64_t *>(g_stage + kHeadersOff);
    int64_t *h_tile0 = reinterpret_cast<int64_t *>(g_stage + kTile0Off);
    KernelArgs *h_args = reinterpret_cast<KernelArgs *>(g_stage + kArgsOff);
    unsigned long long *d_counters = reinterpret_cast<unsigned long long *>(S.scratch + kCountersOff);
    int used = 0;
    int first[kKinds] = {};
    gmle::LaunchShape shape[kKinds] = {};
    for (int kind = 0; kind < kKinds; kind++) {
        int cnt = 0;
        int64_t rois = 0;
        for (int k = 0; k < ngroups; k++)
            if (groups[k].n > 0 && gmle_rt::kind_of(groups[k].desc) == kind) {
                g_order[cnt++] = k;
                rois += groups[k].n;
            }
        first[kind] = used;
        if (cnt == 0) continue;
        const gmle_fit_desc &d0 = groups[g_order[0]].desc;
        const bool scmos = d0.camera != GMLE_CAMERA_POISSON;
        const gmle_rt::Tuning t = gmle_rt::default_tuning(S.num_sms, d0.model, d0.box, scmos, rois);
        int64_t tiles = 0;
        for (int q = 0; q < cnt; q++) {
            const gmle_group &G = groups[g_order[q]];
            KernelArgs &A = h_args[used + q];
            std::memset(&A, 0, sizeof A);
            A.data = G.data;
            A.xc = G.x_corners;
            A.yc = G.y_corners;
            A.n = G.n;
            A.var = variance;
            A.gain = gain;
            A.offset = offset;
            A.ny = variance ? ny : 0;
            A.nx = variance ? nx : 0;
            A.adu = G.desc.camera == GMLE_CAMERA_SCMOS_ADU;
            A.iterations = G.desc.iterations;
            A.tpr = t.tpr;
            A.sqrt2pi = sqrtf(2.0f * (float)3.14159265358979323846);
            std::memcpy(A.psf, G.desc.psf, sizeof A.psf);
            std::memcpy(A.lower, G.desc.lower, sizeof A.lower);
            std::memcpy(A.upper, G.desc.upper, sizeof A.upper);
            std::memcpy(A.max_step, G.desc.max_step, sizeof A.max_step);
            A.params = G.params;
            A.crlb = G.crlb;
            A.llr = G.llr;
            A.flags = G.flags;
            A.bad_corners = d_counters + kBadCounter;
            h_tile0[used + q] = tiles;
            tiles += (G.n + t.rois_per_block - 1) / t.rois_per_block;
        }
        h_headers[2 * kind] = cnt;
        h_headers[2 * kind + 1] = tiles;
        const int bps = gmle::table_blocks_per_sm(d0.model, d0.box, scmos, t.tpr, t.rois_per_block);
        if (bps <= 0)
            return report(err, err_len, GMLE_CUDA_ERROR,
                          "no resident block for model %d box %d (tpr %d, %d ROIs)%s%s", d0.model,
                          d0.box, t.tpr, t.rois_per_block, bps < 0 ? ": " : "",
                          bps < 0 ? cudaGetErrorString((cudaError_t)-bps) : "");
        shape[kind] = gmle::LaunchShape{t.tpr, t.rois_per_block,
                                        std::min<int64_t>((int64_t)S.num_sms * bps, tiles)};
        used += cnt;
    }
    if (used == 0) return GMLE_OK;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t image = kArgsOff + sizeof(KernelArgs) * (size_t)used;
    for (size_t off = 0; off < image; off += kChunkBytes) {
        const size_t b = std::min<size_t>(kChunkBytes, image - off);
        g_chunk.offset = (uint32_t)off;
        g_chunk.bytes = (uint32_t)b;
        std::memcpy(g_chunk.data, g_stage + off, b);
        write_scratch<<<1, 256, 0, s>>>(g_chunk);
        e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_report(err, err_len, e, "group table write");
    }
    for (int kind = 0; kind < kKinds; kind++) {
        if (h_headers[2 * kind] == 0) continue;
        const KernelArgs &A0 = h_args[first[kind]];
        const int model = (kind / gmle::kNumBoxes) % 4;
        const int box = gmle::box_of_index(kind % gmle::kNumBoxes);
        const bool scmos = kind >= kKinds / 2;
        gmle::TileTable t;
        t.header = reinterpret_cast<const int64_t *>(S.scratch + kHeadersOff) + 2 * kind;
        t.groups = reinterpret_cast<const KernelArgs *>(S.scratch + kArgsOff) + first[kind];
        t.tiles = nullptr;
        t.tile0 = reinterpret_cast<const int64_t *>(S.scratch + kTile0Off) + first[kind];
        t.counter = d_counters + kind;
        KernelArgs a;
        std::memset(&a, 0, sizeof a);
        a.tpr = A0.tpr;
        e = gmle::launch_fit(model, box, scmos, a, t, shape[kind], s);
        if (e != cudaSuccess) return cuda_report(err, err_len, e, "table launch");
    }
    return GMLE_OK;
}
