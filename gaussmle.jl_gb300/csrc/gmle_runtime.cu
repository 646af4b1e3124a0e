// gmle_runtime.cu - the C ABI of libgaussmle_sm100a.so (include/gaussmle_gb300.h).
//
// Host runtime around the fit kernels: device context, resident calibration
// maps, launch-shape selection, and the host-buffer fit pipeline that replaces
// the per-batch allocate / copyto! / launch / synchronize / copy-back loop of
// GaussMLE.fit (src/interface.jl:220-262, :336-369, :423-456).  Each context
// owns three CUDA streams (H2D copies, kernels, D2H copies) and two pipeline
// slots, so that chunk k+1 is copied in while chunk k is fitted and chunk k-1
// is copied out.  Device and pinned buffers grow on demand and are reused by
// later calls; nothing the library allocates is handed to the caller.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "gmle_internal.h"

using gmle::KernelArgs;
using namespace gmle_rt;

namespace gmle_rt {

int nparams(int model) { return model == 0 ? 4 : (model == 2 ? 6 : 5); }

gmle_status fail(gmle_ctx *ctx, gmle_status st, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    return st;
}

gmle_status cuda_fail(gmle_ctx *ctx, cudaError_t e, const char *what)
{
    if (e == cudaErrorMemoryAllocation)
        return fail(ctx, GMLE_OUT_OF_MEMORY, "%s: %s", what, cudaGetErrorString(e));
    return fail(ctx, GMLE_CUDA_ERROR, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what) GMLE_CK(call, what)

gmle_status check_desc(gmle_ctx *ctx, const gmle_fit_desc *d)
{
    if (!d) return fail(ctx, GMLE_INVALID_ARG, "desc is NULL");
    if (d->model < 0 || d->model > 3)
        return fail(ctx, GMLE_UNSUPPORTED_MODEL, "unknown model id %d", d->model);
    if (!gmle::box_supported(d->box) && !gmle::generic_box(d->box))
        return fail(ctx, GMLE_UNSUPPORTED_BOX, "box size %d: ROIs of %d..%d pixels are supported",
                    d->box, gmle::kMinBox, gmle::kGenericMaxBox);
    if (gmle::generic_box(d->box) && d->method != GMLE_METHOD_NEWTON)
        return fail(ctx, GMLE_UNSUPPORTED_BOX,
                    "box size %d: the full-Hessian method takes boxes %d..%d", d->box,
                    gmle::kMinBox, gmle::kMaxBox);
    if (d->iterations < 0) return fail(ctx, GMLE_INVALID_ARG, "iterations < 0");
    if (d->camera < 0 || d->camera > 2)
        return fail(ctx, GMLE_INVALID_ARG, "unknown camera id %d", d->camera);
    if (d->method != GMLE_METHOD_NEWTON && d->method != GMLE_METHOD_FISHER_LM)
        return fail(ctx, GMLE_INVALID_ARG, "unknown method id %d", d->method);
    if (d->camera != GMLE_CAMERA_POISSON) {
        if (!ctx->d_var) return fail(ctx, GMLE_INVALID_ARG, "sCMOS fit without calibration maps");
        if (d->camera == GMLE_CAMERA_SCMOS_ADU && (!ctx->d_gain || !ctx->d_offset))
            return fail(ctx, GMLE_INVALID_ARG, "ADU fit needs gain and offset maps");
    }
    if (d->model == GMLE_MODEL_XYNB && !(d->psf[0] > 0.f))
        return fail(ctx, GMLE_INVALID_ARG, "GaussianXYNB sigma must be > 0");
    if (d->model == GMLE_MODEL_ASTIG && (!(d->psf[0] > 0.f) || !(d->psf[1] > 0.f) || d->psf[7] == 0.f))
        return fail(ctx, GMLE_INVALID_ARG, "astigmatic sigma0 must be > 0 and d != 0");
    return GMLE_OK;
}

}  // namespace gmle_rt

namespace gmle_rt {

// Launch shape: enough threads to fill the GPU (threads per ROI grows for small
// batches), and ROIs per block bounded by shared memory.
Tuning default_tuning(int num_sms, int model, int box, bool scmos, int64_t n)
{
    // Resident ROIs per SM are bounded by shared memory; threads per ROI grow
    // until about 16 warps per SM are resident and the batch fills the GPU.
    const size_t per_roi = gmle::smem_bytes(model, box, scmos, 1, 1);
    const int64_t rois_per_sm = (int64_t)((200 * 1024) / per_roi);
    const int64_t want_threads_sm = 512;
    int tpr = 1;
    if (rois_per_sm < want_threads_sm || n < (int64_t)num_sms * want_threads_sm) tpr = 4;
    // one thread per ROI with sCMOS data: blocks of 4 warps use the tensor
    // memory that holds the variance tiles fully
    int rpb = tpr == 1 ? (scmos ? 128 : 32) : 128 / tpr;
    while (rpb * tpr > 32 && gmle::smem_bytes(model, box, scmos, tpr, rpb) > 100 * 1024) rpb /= 2;
    if (rpb * tpr < 32) rpb = 32 / tpr;
    return {tpr, rpb};
}

}  // namespace gmle_rt

namespace gmle_rt {

Tuning pick_tuning(gmle_ctx *ctx, const gmle_fit_desc *d, int64_t n)
{
    const bool scmos = d->camera != GMLE_CAMERA_POISSON;
    if (gmle::generic_box(d->box)) return {1, gmle::generic_rois_per_block(d->box, scmos)};
    auto it = ctx->tuning.find({d->model, d->box, (int)scmos});
    Tuning t = it != ctx->tuning.end() ? it->second
                                       : default_tuning(ctx->num_sms, d->model, d->box, scmos, n);
    if (d->method == GMLE_METHOD_FISHER_LM && t.tpr != 1) {
        // the full-Hessian method runs one thread per ROI; 128-thread blocks
        // use the tensor memory of sCMOS variance tiles fully
        t.tpr = 1;
        t.rois_per_block = scmos ? 128 : 64;
    }
    return t;
}

KernelArgs make_args(gmle_ctx *ctx, const gmle_fit_desc *d, const float *data, const int32_t *xc,
                     const int32_t *yc, int64_t n, float *params, float *crlb, float *llr,
                     uint8_t *flags, int tpr)
{
    KernelArgs a;
    std::memset(&a, 0, sizeof a);
    a.data = data;
    a.xc = xc;
    a.yc = yc;
    a.n = n;
    a.var = ctx->d_var;
    a.gain = ctx->d_gain;
    a.offset = ctx->d_offset;
    a.ny = ctx->ny;
    a.nx = ctx->nx;
    a.adu = d->camera == GMLE_CAMERA_SCMOS_ADU;
    a.iterations = d->iterations;
    a.tpr = tpr;
    // sqrt(two * one(T) * pi) in Float32, as src/gausslib/baselibrary.jl:26 evaluates it
    a.sqrt2pi = sqrtf(2.0f * (float)3.14159265358979323846);
    std::memcpy(a.psf, d->psf, sizeof a.psf);
    std::memcpy(a.lower, d->lower, sizeof a.lower);
    std::memcpy(a.upper, d->upper, sizeof a.upper);
    std::memcpy(a.max_step, d->max_step, sizeof a.max_step);
    a.params = params;
    a.crlb = crlb;
    a.llr = llr;
    a.flags = flags;
    a.bad_corners = ctx->d_bad;
    return a;
}

}  // namespace gmle_rt

namespace {

cudaError_t launch(gmle_ctx *ctx, const gmle_fit_desc *d, const KernelArgs &a, int rpb,
                   cudaStream_t s)
{
    const bool scmos = d->camera != GMLE_CAMERA_POISSON;
    ctx->launches++;
    if (gmle::generic_box(d->box)) return gmle::launch_fit_generic(d->model, d->box, scmos, a, s);
    gmle::LaunchShape shape{a.tpr, rpb, 0};
    shape.lm = d->method == GMLE_METHOD_FISHER_LM;
    return gmle::launch_fit(d->model, d->box, scmos, a, gmle::TileTable{}, shape, s);
}

bool is_pinned(const void *p)
{
    cudaPointerAttributes attr;
    if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeHost;
}

void free_slot(Slot &s)
{
    cudaFree(s.data);
    cudaFree(s.xc);
    cudaFree(s.yc);
    cudaFree(s.params);
    cudaFree(s.crlb);
    cudaFree(s.llr);
    cudaFree(s.flags);
    cudaFreeHost(s.h_data);
    cudaFreeHost(s.h_params);
    cudaFreeHost(s.h_crlb);
    cudaFreeHost(s.h_llr);
    cudaFreeHost(s.h_flags);
    if (s.h2d_done) cudaEventDestroy(s.h2d_done);
    if (s.fit_done) cudaEventDestroy(s.fit_done);
    if (s.d2h_done) cudaEventDestroy(s.d2h_done);
    s = Slot();
}

gmle_status ensure_slot(gmle_ctx *ctx, Slot &s, int64_t rois, int64_t b2, bool need_pinned)
{
    if (!s.h2d_done) {
        CK(cudaEventCreateWithFlags(&s.h2d_done, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&s.fit_done, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&s.d2h_done, cudaEventDisableTiming), "cudaEventCreate");
    }
    if (s.cap_rois < rois || s.cap_b2 < b2) {
        cudaFree(s.data); cudaFree(s.xc); cudaFree(s.yc);
        cudaFree(s.params); cudaFree(s.crlb); cudaFree(s.llr); cudaFree(s.flags);
        s.data = nullptr; s.xc = s.yc = nullptr; s.params = s.crlb = s.llr = nullptr; s.flags = nullptr;
        s.cap_rois = s.cap_b2 = 0;
        CK(cudaMalloc(&s.data, sizeof(float) * rois * b2), "cudaMalloc(data)");
        CK(cudaMalloc(&s.xc, sizeof(int32_t) * rois), "cudaMalloc(corners)");
        CK(cudaMalloc(&s.yc, sizeof(int32_t) * rois), "cudaMalloc(corners)");
        CK(cudaMalloc(&s.params, sizeof(float) * rois * 6), "cudaMalloc(params)");
        CK(cudaMalloc(&s.crlb, sizeof(float) * rois * 6), "cudaMalloc(crlb)");
        CK(cudaMalloc(&s.llr, sizeof(float) * rois), "cudaMalloc(llr)");
        CK(cudaMalloc(&s.flags, rois), "cudaMalloc(flags)");
        s.cap_rois = rois;
        s.cap_b2 = b2;
    }
    if (need_pinned && (s.h_cap_rois < rois || s.h_cap_b2 < b2)) {
        cudaFreeHost(s.h_data); cudaFreeHost(s.h_params); cudaFreeHost(s.h_crlb);
        cudaFreeHost(s.h_llr); cudaFreeHost(s.h_flags);
        s.h_data = nullptr; s.h_params = s.h_crlb = s.h_llr = nullptr; s.h_flags = nullptr;
        s.h_cap_rois = s.h_cap_b2 = 0;
        CK(cudaMallocHost(&s.h_data, sizeof(float) * rois * b2), "cudaMallocHost(data)");
        CK(cudaMallocHost(&s.h_params, sizeof(float) * rois * 6), "cudaMallocHost(params)");
        CK(cudaMallocHost(&s.h_crlb, sizeof(float) * rois * 6), "cudaMallocHost(crlb)");
        CK(cudaMallocHost(&s.h_llr, sizeof(float) * rois), "cudaMallocHost(llr)");
        CK(cudaMallocHost(&s.h_flags, rois), "cudaMallocHost(flags)");
        s.h_cap_rois = rois;
        s.h_cap_b2 = b2;
    }
    return GMLE_OK;
}

// Copy a finished slot's pinned outputs to the caller's pageable buffers.
gmle_status flush_slot(gmle_ctx *ctx, Slot &s)
{
    if (!s.pending) return GMLE_OK;
    CK(cudaEventSynchronize(s.d2h_done), "cudaEventSynchronize");
    std::memcpy(s.dst_params, s.h_params, sizeof(float) * s.pend_rois * s.pend_p);
    std::memcpy(s.dst_crlb, s.h_crlb, sizeof(float) * s.pend_rois * s.pend_p);
    std::memcpy(s.dst_llr, s.h_llr, sizeof(float) * s.pend_rois);
    if (s.dst_flags) std::memcpy(s.dst_flags, s.h_flags, s.pend_rois);
    s.pending = false;
    return GMLE_OK;
}

gmle_status check_corners_host(gmle_ctx *ctx, const gmle_fit_desc *d, const int32_t *xc,
                               const int32_t *yc, int64_t n)
{
    if (d->camera == GMLE_CAMERA_POISSON) return GMLE_OK;
    if (!xc || !yc) return fail(ctx, GMLE_INVALID_ARG, "sCMOS fit needs ROI corners");
    for (int64_t k = 0; k < n; k++) {
        const int64_t x = xc[k], y = yc[k];
        if (x < 1 || y < 1 || x + d->box - 1 > ctx->nx || y + d->box - 1 > ctx->ny)
            return fail(ctx, GMLE_INVALID_ARG,
                        "ROI %lld: corner (x=%lld, y=%lld) puts the %dx%d box outside the %dx%d "
                        "calibration map",
                        (long long)k, (long long)x, (long long)y, d->box, d->box, ctx->ny, ctx->nx);
    }
    return GMLE_OK;
}

}  // namespace

extern "C" {

int gmle_abi_version(void) { return GMLE_ABI_VERSION; }

gmle_status gmle_create(gmle_ctx **out, int device_ordinal)
{
    if (!out) return GMLE_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return GMLE_NO_DEVICE;
    }
    if (device_ordinal < 0 || device_ordinal >= count) return GMLE_NO_DEVICE;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device_ordinal) != cudaSuccess) return GMLE_NO_DEVICE;
    // The kernels are built for sm_103a only.
    if (prop.major != 10 || prop.minor != 3) return GMLE_NO_DEVICE;
    gmle_ctx *ctx = new gmle_ctx();
    ctx->device = device_ordinal;
    ctx->num_sms = prop.multiProcessorCount;
    cudaSetDevice(device_ordinal);
    if (cudaStreamCreateWithFlags(&ctx->s_fit, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->s_h2d, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->s_d2h, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->d_bad, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMemset(ctx->d_bad, 0, sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        gmle_destroy(ctx);
        return GMLE_CUDA_ERROR;
    }
    *out = ctx;
    return GMLE_OK;
}

void gmle_destroy(gmle_ctx *ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->s_fit) cudaStreamSynchronize(ctx->s_fit);
    if (ctx->s_h2d) cudaStreamSynchronize(ctx->s_h2d);
    if (ctx->s_d2h) cudaStreamSynchronize(ctx->s_d2h);
    server_destroy(ctx);
    for (Slot &s : ctx->slots) free_slot(s);
    free_mixed_set(ctx->mixed);
    cudaFree(ctx->d_var);
    cudaFree(ctx->d_gain);
    cudaFree(ctx->d_offset);
    cudaFree(ctx->d_bad);
    cudaFree(ctx->d_pv);
    if (ctx->s_fit) cudaStreamDestroy(ctx->s_fit);
    if (ctx->s_h2d) cudaStreamDestroy(ctx->s_h2d);
    if (ctx->s_d2h) cudaStreamDestroy(ctx->s_d2h);
    delete ctx;
}

const char *gmle_last_error(const gmle_ctx *ctx)
{
    if (!ctx) return "no context";
    return ctx->err.c_str();
}

gmle_status gmle_set_calibration(gmle_ctx *ctx, const float *variance, const float *gain,
                                 const float *offset, int32_t ny, int32_t nx)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!variance || ny <= 0 || nx <= 0)
        return fail(ctx, GMLE_INVALID_ARG, "variance map and positive ny, nx are required");
    if ((gain == nullptr) != (offset == nullptr))
        return fail(ctx, GMLE_INVALID_ARG, "gain and offset maps come together");
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->s_fit), "cudaStreamSynchronize");
    cudaFree(ctx->d_var);
    cudaFree(ctx->d_gain);
    cudaFree(ctx->d_offset);
    ctx->d_var = ctx->d_gain = ctx->d_offset = nullptr;
    ctx->ny = ctx->nx = 0;
    const size_t bytes = sizeof(float) * (size_t)ny * (size_t)nx;
    CK(cudaMalloc(&ctx->d_var, bytes), "cudaMalloc(variance)");
    CK(cudaMemcpy(ctx->d_var, variance, bytes, cudaMemcpyHostToDevice), "upload variance");
    if (gain) {
        CK(cudaMalloc(&ctx->d_gain, bytes), "cudaMalloc(gain)");
        CK(cudaMalloc(&ctx->d_offset, bytes), "cudaMalloc(offset)");
        CK(cudaMemcpy(ctx->d_gain, gain, bytes, cudaMemcpyHostToDevice), "upload gain");
        CK(cudaMemcpy(ctx->d_offset, offset, bytes, cudaMemcpyHostToDevice), "upload offset");
    }
    ctx->ny = ny;
    ctx->nx = nx;
    return GMLE_OK;
}

gmle_status gmle_fit_device(gmle_ctx *ctx, const gmle_fit_desc *desc, const float *d_data,
                            const int32_t *d_x_corners, const int32_t *d_y_corners, int64_t n,
                            float *d_params, float *d_crlb, float *d_llr, uint8_t *d_flags,
                            void *stream)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    gmle_status st = check_desc(ctx, desc);
    if (st != GMLE_OK) return st;
    if (n < 0) return fail(ctx, GMLE_INVALID_ARG, "n < 0");
    if (n == 0) return GMLE_OK;
    if (!d_data || !d_params || !d_crlb || !d_llr)
        return fail(ctx, GMLE_INVALID_ARG, "data and output pointers are required");
    if (desc->camera != GMLE_CAMERA_POISSON && (!d_x_corners || !d_y_corners))
        return fail(ctx, GMLE_INVALID_ARG, "sCMOS fit needs ROI corners");
    cudaSetDevice(ctx->device);
    const Tuning t = pick_tuning(ctx, desc, n);
    KernelArgs a = make_args(ctx, desc, d_data, d_x_corners, d_y_corners, n, d_params, d_crlb,
                             d_llr, d_flags, t.tpr);
    CK(launch(ctx, desc, a, t.rois_per_block, (cudaStream_t)stream), "fit kernel launch");
    return GMLE_OK;
}

gmle_status gmle_fit_device_errors(gmle_ctx *ctx, int64_t *count)
{
    if (!ctx || !count) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    cudaSetDevice(ctx->device);
    unsigned long long v = 0;
    CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
    CK(cudaMemcpy(&v, ctx->d_bad, sizeof v, cudaMemcpyDeviceToHost), "read error counter");
    CK(cudaMemset(ctx->d_bad, 0, sizeof v), "reset error counter");
    *count = (int64_t)v;
    return GMLE_OK;
}

gmle_status gmle_fit(gmle_ctx *ctx, const gmle_fit_desc *desc, const float *data,
                     const int32_t *x_corners, const int32_t *y_corners, int64_t n,
                     float *params, float *crlb, float *llr, uint8_t *flags)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    gmle_status st = check_desc(ctx, desc);
    if (st != GMLE_OK) return st;
    if (n < 0) return fail(ctx, GMLE_INVALID_ARG, "n < 0");
    if (n == 0) return GMLE_OK;
    if (!data || !params || !crlb || !llr)
        return fail(ctx, GMLE_INVALID_ARG, "data and output pointers are required");
    st = check_corners_host(ctx, desc, x_corners, y_corners, n);
    if (st != GMLE_OK) return st;
    cudaSetDevice(ctx->device);

    const int P = nparams(desc->model);
    const int64_t b2 = (int64_t)desc->box * desc->box;
    const bool scmos = desc->camera != GMLE_CAMERA_POISSON;
    // Chunk of about 64 MiB of pixel data, at least one full GPU wave.
    int64_t chunk = std::max<int64_t>((int64_t)ctx->num_sms * 1024, (64ll << 20) / (4 * b2));
    chunk = std::min<int64_t>(chunk, n);
    const bool in_pinned = is_pinned(data);
    const bool out_pinned = is_pinned(params) && is_pinned(crlb) && is_pinned(llr) &&
                            (!flags || is_pinned(flags));
    const Tuning t = pick_tuning(ctx, desc, chunk);

    for (Slot &s : ctx->slots) {
        st = ensure_slot(ctx, s, chunk, b2, !(in_pinned && out_pinned));
        if (st != GMLE_OK) return st;
    }
    int k = 0;
    for (int64_t off = 0; off < n; off += chunk, k ^= 1) {
        Slot &s = ctx->slots[k];
        const int64_t m = std::min(chunk, n - off);
        // The slot's previous chunk must be out before its buffers are reused.
        st = flush_slot(ctx, s);
        if (st != GMLE_OK) return st;
        CK(cudaStreamWaitEvent(ctx->s_h2d, s.d2h_done, 0), "cudaStreamWaitEvent");
        const float *src = data + off * b2;
        if (!in_pinned) {
            CK(cudaEventSynchronize(s.h2d_done), "cudaEventSynchronize");
            std::memcpy(s.h_data, src, sizeof(float) * m * b2);
            src = s.h_data;
        }
        CK(cudaMemcpyAsync(s.data, src, sizeof(float) * m * b2, cudaMemcpyHostToDevice, ctx->s_h2d),
           "H2D data");
        if (scmos) {
            CK(cudaMemcpyAsync(s.xc, x_corners + off, sizeof(int32_t) * m, cudaMemcpyHostToDevice,
                               ctx->s_h2d), "H2D corners");
            CK(cudaMemcpyAsync(s.yc, y_corners + off, sizeof(int32_t) * m, cudaMemcpyHostToDevice,
                               ctx->s_h2d), "H2D corners");
        }
        CK(cudaEventRecord(s.h2d_done, ctx->s_h2d), "cudaEventRecord");
        CK(cudaStreamWaitEvent(ctx->s_fit, s.h2d_done, 0), "cudaStreamWaitEvent");
        KernelArgs a = make_args(ctx, desc, s.data, scmos ? s.xc : nullptr, scmos ? s.yc : nullptr,
                                 m, s.params, s.crlb, s.llr, s.flags, t.tpr);
        CK(launch(ctx, desc, a, t.rois_per_block, ctx->s_fit), "fit kernel launch");
        CK(cudaEventRecord(s.fit_done, ctx->s_fit), "cudaEventRecord");
        CK(cudaStreamWaitEvent(ctx->s_d2h, s.fit_done, 0), "cudaStreamWaitEvent");
        float *op = out_pinned ? params + off * P : s.h_params;
        float *oc = out_pinned ? crlb + off * P : s.h_crlb;
        float *ol = out_pinned ? llr + off : s.h_llr;
        uint8_t *of = out_pinned ? (flags ? flags + off : nullptr) : s.h_flags;
        CK(cudaMemcpyAsync(op, s.params, sizeof(float) * m * P, cudaMemcpyDeviceToHost, ctx->s_d2h),
           "D2H params");
        CK(cudaMemcpyAsync(oc, s.crlb, sizeof(float) * m * P, cudaMemcpyDeviceToHost, ctx->s_d2h),
           "D2H crlb");
        CK(cudaMemcpyAsync(ol, s.llr, sizeof(float) * m, cudaMemcpyDeviceToHost, ctx->s_d2h),
           "D2H llr");
        if (of)
            CK(cudaMemcpyAsync(of, s.flags, m, cudaMemcpyDeviceToHost, ctx->s_d2h), "D2H flags");
        CK(cudaEventRecord(s.d2h_done, ctx->s_d2h), "cudaEventRecord");
        if (!out_pinned) {
            s.pending = true;
            s.dst_params = params + off * P;
            s.dst_crlb = crlb + off * P;
            s.dst_llr = llr + off;
            s.dst_flags = flags ? flags + off : nullptr;
            s.pend_rois = m;
            s.pend_p = P;
        }
    }
    for (Slot &s : ctx->slots) {
        st = flush_slot(ctx, s);
        if (st != GMLE_OK) return st;
    }
    CK(cudaStreamSynchronize(ctx->s_d2h), "cudaStreamSynchronize");
    CK(cudaStreamSynchronize(ctx->s_fit), "cudaStreamSynchronize");
    return GMLE_OK;
}

gmle_status gmle_get_tuning(gmle_ctx *ctx, int32_t model, int32_t box, int32_t camera,
                            int32_t *threads_per_roi, int32_t *rois_per_block)
{
    if (!ctx || !threads_per_roi || !rois_per_block) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const bool scmos = camera != GMLE_CAMERA_POISSON;
    auto it = ctx->tuning.find({model, box, (int)scmos});
    Tuning t = it != ctx->tuning.end() ? it->second
                                       : default_tuning(ctx->num_sms, model, box, scmos, 1ll << 40);
    *threads_per_roi = t.tpr;
    *rois_per_block = t.rois_per_block;
    return GMLE_OK;
}

gmle_status gmle_set_tuning(gmle_ctx *ctx, int32_t model, int32_t box, int32_t camera,
                            int32_t threads_per_roi, int32_t rois_per_block)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int tpr = threads_per_roi;
    if (tpr == 0 && rois_per_block == 0) {  // forget the entry: size-based default again
        ctx->tuning.erase({model, box, (int)(camera != GMLE_CAMERA_POISSON)});
        return GMLE_OK;
    }
    if (model < 0 || model > 3) return fail(ctx, GMLE_UNSUPPORTED_MODEL, "unknown model");
    if (!gmle::box_supported(box))
        return fail(ctx, GMLE_UNSUPPORTED_BOX, "box %d has no launch-shape choice (3..16)", box);
    if (!gmle::tpr_supported(tpr, box))
        return fail(ctx, GMLE_INVALID_ARG,
                    "threads_per_roi must be 1, 2, 4, or 8 (2 and 8: odd boxes 5..15 only)");
    const bool scmos = camera != GMLE_CAMERA_POISSON;
    const int threads = tpr * rois_per_block;
    if (rois_per_block < 1 || threads > (tpr == 1 ? gmle::kMaxThreadsR1 : 256) || threads % 32)
        return fail(ctx, GMLE_INVALID_ARG,
                    "threads_per_roi * rois_per_block must be a multiple of 32, at most 256 "
                    "(64 with one thread per ROI)");
    if (gmle::smem_bytes(model, box, scmos, tpr, rois_per_block) > 227 * 1024)
        return fail(ctx, GMLE_INVALID_ARG, "launch shape needs more than 227 KiB shared memory");
    ctx->tuning[{model, box, (int)scmos}] = {tpr, rois_per_block};
    return GMLE_OK;
}

int64_t gmle_kernel_launches(const gmle_ctx *ctx) { return ctx ? ctx->launches : 0; }

gmle_status gmle_autotune(gmle_ctx *ctx, const gmle_fit_desc *desc, const float *d_data,
                          const int32_t *d_x_corners, const int32_t *d_y_corners, int64_t n,
                          float *d_params, float *d_crlb, float *d_llr, uint8_t *d_flags,
                          int32_t *threads_per_roi, int32_t *rois_per_block, float *ms_per_fit)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    gmle_status st = check_desc(ctx, desc);
    if (st != GMLE_OK) return st;
    if (n <= 0 || !d_data || !d_params || !d_crlb || !d_llr)
        return fail(ctx, GMLE_INVALID_ARG, "autotune needs a non-empty device batch");
    if (desc->camera != GMLE_CAMERA_POISSON && (!d_x_corners || !d_y_corners))
        return fail(ctx, GMLE_INVALID_ARG, "sCMOS fit needs ROI corners");
    cudaSetDevice(ctx->device);
    const bool scmos = desc->camera != GMLE_CAMERA_POISSON;
    if (gmle::generic_box(desc->box)) {
        // one launch shape: the run-time-box kernel's
        const Tuning t = pick_tuning(ctx, desc, n);
        cudaEvent_t e0, e1;
        CK(cudaEventCreate(&e0), "cudaEventCreate");
        CK(cudaEventCreate(&e1), "cudaEventCreate");
        KernelArgs a = make_args(ctx, desc, d_data, d_x_corners, d_y_corners, n, d_params,
                                 d_crlb, d_llr, d_flags, 1);
        cudaError_t e = cudaEventRecord(e0, ctx->s_fit);
        if (e == cudaSuccess) e = launch(ctx, desc, a, t.rois_per_block, ctx->s_fit);
        if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->s_fit);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "autotune launch");
        if (threads_per_roi) *threads_per_roi = 1;
        if (rois_per_block) *rois_per_block = t.rois_per_block;
        if (ms_per_fit) *ms_per_fit = ms;
        return GMLE_OK;
    }
    // shapes are kept per (model, box, camera family) and timed with the
    // reference's method, which runs in every shape
    gmle_fit_desc dn = *desc;
    dn.method = GMLE_METHOD_NEWTON;
    desc = &dn;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "cudaEventCreate");
    CK(cudaEventCreate(&e1), "cudaEventCreate");
    Tuning best{0, 0};
    float best_ms = 1e30f;
    // threads per block: powers of two, and for one thread per ROI also 96
    // (three warps: two such blocks of large sCMOS ROIs fit where one of four
    // warps does)
    static const int kThreads[] = {32, 64, 96, 128, 256};
    for (int tpr : {1, 2, 4, 8}) {
        if (!gmle::tpr_supported(tpr, desc->box)) continue;
        for (int threads : kThreads) {
            if (threads > (tpr == 1 ? gmle::kMaxThreadsR1 : 256)) continue;
            if (tpr > 1 && threads == 96) continue;
            const int rpb = threads / tpr;
            if (rpb < 1 || gmle::smem_bytes(desc->model, desc->box, scmos, tpr, rpb) > 227 * 1024)
                continue;
            KernelArgs a = make_args(ctx, desc, d_data, d_x_corners, d_y_corners, n, d_params,
                                     d_crlb, d_llr, d_flags, tpr);
            // two warm-up launches, then the fastest of four timed one by one:
            // a single average was swayed by clock ramps and by other work on
            // the GPU, and picked slower shapes
            cudaError_t e = launch(ctx, desc, a, rpb, ctx->s_fit);
            if (e == cudaSuccess) e = launch(ctx, desc, a, rpb, ctx->s_fit);
            float ms = 1e30f;
            for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
                e = cudaEventRecord(e0, ctx->s_fit);
                if (e == cudaSuccess) e = launch(ctx, desc, a, rpb, ctx->s_fit);
                if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->s_fit);
                if (e == cudaSuccess) e = cudaEventSynchronize(e1);
                float t = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
                if (e == cudaSuccess) ms = std::min(ms, t);
            }
            if (e != cudaSuccess) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                return cuda_fail(ctx, e, "autotune launch");
            }
            if (ms < best_ms) {
                best_ms = ms;
                best = {tpr, rpb};
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->tuning[{desc->model, desc->box, (int)scmos}] = best;
    if (threads_per_roi) *threads_per_roi = best.tpr;
    if (rois_per_block) *rois_per_block = best.rois_per_block;
    if (ms_per_fit) *ms_per_fit = best_ms;
    return GMLE_OK;
}

}  // extern "C"

// ---- mixed batches: one persistent table launch per (family, model, box) ----------

namespace gmle_rt {

namespace {

void free_table(TableBufs &b)
{
    if (b.reuse) cudaEventSynchronize(b.reuse);
    cudaFreeHost(b.h_base);
    cudaFree(b.d_base);
    cudaFree(b.d_counter);
    if (b.reuse) cudaEventDestroy(b.reuse);
    if (b.used) cudaEventDestroy(b.used);
    b = TableBufs();
}

// Room for `groups` groups and `tiles` tiles (grown by half again when short).
gmle_status ensure_table(gmle_ctx *ctx, TableBufs &b, int64_t groups, int64_t tiles,
                         bool device_copy)
{
    if (b.in_pool) {  // leaving the pool: a table of its own
        b.h_base = nullptr;
        b.cap_groups = b.cap_tiles = 0;
        b.in_pool = false;
    }
    if (!b.reuse) {
        CK(cudaEventCreateWithFlags(&b.reuse, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&b.used, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaMalloc(&b.d_counter, sizeof(unsigned long long)), "cudaMalloc(tile counter)");
    }
    if (b.cap_groups >= groups && b.cap_tiles >= tiles) return GMLE_OK;
    CK(cudaEventSynchronize(b.reuse), "cudaEventSynchronize");
    CK(cudaEventSynchronize(b.used), "cudaEventSynchronize");
    cudaFreeHost(b.h_base);
    cudaFree(b.d_base);
    b.h_base = b.d_base = nullptr;
    b.cap_groups = std::max<int64_t>({64, groups, b.cap_groups + b.cap_groups / 2});
    b.cap_tiles = std::max<int64_t>({1024, tiles, b.cap_tiles + b.cap_tiles / 2});
    CK(cudaMallocHost(&b.h_base, b.bytes()), "cudaMallocHost(group table)");
    if (device_copy) CK(cudaMalloc(&b.d_base, b.bytes()), "cudaMalloc(group table)");
    return GMLE_OK;
}

}  // namespace

gmle_status validate_groups(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups)
{
    for (int k = 0; k < ngroups; k++) {
        const gmle_group &G = groups[k];
        gmle_status st = check_desc(ctx, &G.desc);
        if (st != GMLE_OK) return st;
        if (!gmle::box_supported(G.desc.box))
            return fail(ctx, GMLE_UNSUPPORTED_BOX,
                        "group %d: box size %d: mixed batches and serving take boxes %d..%d "
                        "(larger ROIs: gmle_fit or gmle_fit_device)", k, G.desc.box,
                        gmle::kMinBox, gmle::kMaxBox);
        if (G.n < 0) return fail(ctx, GMLE_INVALID_ARG, "group %d: n < 0", k);
        if (G.n > 0 && (!G.data || !G.params || !G.crlb || !G.llr))
            return fail(ctx, GMLE_INVALID_ARG, "group %d: data and output pointers are required", k);
        if (G.n > 0 && G.desc.camera != GMLE_CAMERA_POISSON && (!G.x_corners || !G.y_corners))
            return fail(ctx, GMLE_INVALID_ARG, "group %d: sCMOS fit needs ROI corners", k);
        if (G.n > 0x7fffffffLL * 32)
            return fail(ctx, GMLE_INVALID_ARG, "group %d: more ROIs than a table indexes", k);
        if (G.desc.method != GMLE_METHOD_NEWTON)
            return fail(ctx, GMLE_INVALID_ARG,
                        "group %d: method %d runs through gmle_fit and gmle_fit_device only", k,
                        G.desc.method);
    }
    return GMLE_OK;
}

gmle_status init_mixed_set(gmle_ctx *ctx, MixedSet &m)
{
    if (m.ev_fork) return GMLE_OK;
    for (int c = 0; c < kForks; c++) {
        CK(cudaStreamCreateWithFlags(&m.fork[c], cudaStreamNonBlocking), "cudaStreamCreate");
        CK(cudaEventCreateWithFlags(&m.ev_join[c], cudaEventDisableTiming), "cudaEventCreate");
    }
    CK(cudaEventCreateWithFlags(&m.ev_fork, cudaEventDisableTiming), "cudaEventCreate");
    return GMLE_OK;
}

void free_mixed_set(MixedSet &m)
{
    for (TableBufs &b : m.tables) {
        if (b.in_pool) b.h_base = nullptr;
        free_table(b);
    }
    if (m.pool) cudaFreeHost(m.pool);
    for (int c = 0; c < kForks; c++) {
        if (m.fork[c]) {
            cudaStreamSynchronize(m.fork[c]);
            cudaStreamDestroy(m.fork[c]);
        }
        if (m.ev_join[c]) cudaEventDestroy(m.ev_join[c]);
    }
    if (m.ev_fork) cudaEventDestroy(m.ev_fork);
    m = MixedSet();
}

gmle_status plan_mixed(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups, MixedSet &m,
                       MixedPlan &plan, const PlanOptions &opt)
{
    gmle_status st = validate_groups(ctx, groups, ngroups);
    if (st != GMLE_OK) return st;
    plan = MixedPlan();
    m.pool_used = 0;
    std::vector<int> by_kind[kKinds];
    int64_t rois[kKinds] = {};
    for (int k = 0; k < ngroups; k++) {
        const gmle_group &G = groups[k];
        if (G.n <= 0) continue;
        if (opt.allow_plain && G.n >= kPlainGroupRois) {
            plan.plain.push_back(G);
            continue;
        }
        const int kind = kind_of(G.desc);
        by_kind[kind].push_back(k);
        rois[kind] += G.n;
    }
    for (int kind = 0; kind < kKinds; kind++) {
        if (by_kind[kind].empty()) continue;
        const gmle_fit_desc &d0 = groups[by_kind[kind][0]].desc;
        TableLaunch L;
        L.kind = kind;
        L.model = d0.model;
        L.box = d0.box;
        L.scmos = d0.camera != GMLE_CAMERA_POISSON;
        const Tuning t = pick_tuning(ctx, &d0, opt.shape_rois > 0 ? opt.shape_rois : rois[kind]);
        const int rpb = t.rois_per_block;
        int64_t tiles = 0;
        for (int k : by_kind[kind]) tiles += (groups[k].n + rpb - 1) / rpb;
        TableBufs &b = m.tables[kind];
        const int64_t ng = (int64_t)by_kind[kind].size();
        const size_t need = (kTableHeader + sizeof(KernelArgs) * (size_t)ng + sizeof(int64_t) * (size_t)tiles +
                             255) & ~size_t(255);
        if (m.pool && m.zero_copy && !opt.persistent && m.pool_used + need <= m.pool_bytes) {
            // the kind's table in the set's pool: no allocation
            if (!b.in_pool && b.h_base) free_table(b);
            b.h_base = m.pool + m.pool_used;
            b.in_pool = true;
            b.cap_groups = ng;
            b.cap_tiles = tiles;
            m.pool_used += need;
        } else {
            st = ensure_table(ctx, b, std::max<int64_t>(ng, opt.reserve_groups),
                              std::max<int64_t>(tiles, opt.reserve_rois / rpb + opt.reserve_groups),
                              !m.zero_copy);
            if (st != GMLE_OK) return st;
        }
        if (!m.zero_copy) CK(cudaEventSynchronize(b.reuse), "cudaEventSynchronize");
        int64_t *hdr = reinterpret_cast<int64_t *>(b.h_base);
        KernelArgs *args = reinterpret_cast<KernelArgs *>(b.h_base + kTableHeader);
        int64_t *map = reinterpret_cast<int64_t *>(b.h_base + b.tiles_off());
        int64_t tile = 0;
        for (size_t q = 0; q < by_kind[kind].size(); q++) {
            const gmle_group &G = groups[by_kind[kind][q]];
            args[q] = make_args(ctx, &G.desc, G.data, G.x_corners, G.y_corners, G.n, G.params,
                                G.crlb, G.llr, G.flags, t.tpr);
            const int64_t nt = (G.n + rpb - 1) / rpb;
            for (int64_t j = 0; j < nt; j++) map[tile + j] = ((int64_t)q << 32) | j;
            tile += nt;
        }
        hdr[0] = (int64_t)by_kind[kind].size();
        hdr[1] = tiles;
        const int bps = gmle::table_blocks_per_sm(L.model, L.box, L.scmos, t.tpr, rpb);
        if (bps <= 0)
            return fail(ctx, GMLE_CUDA_ERROR, "no resident block for model %d box %d (tpr %d, %d ROIs)%s%s",
                        L.model, L.box, t.tpr, rpb, bps < 0 ? ": " : "",
                        bps < 0 ? cudaGetErrorString((cudaError_t)-bps) : "");
        const int64_t full = (int64_t)ctx->num_sms * bps;
        L.persistent = opt.persistent;
        L.shape = gmle::LaunchShape{t.tpr, rpb, !opt.persistent ? tiles
                                                : opt.full_grid ? full
                                                                : std::min(full, tiles)};
        L.groups = hdr[0];
        L.tiles = tiles;
        plan.launches.push_back(L);
    }
    return GMLE_OK;
}

gmle_status upload_plan(gmle_ctx *ctx, MixedSet &m, const MixedPlan &plan, cudaStream_t s,
                        bool record_reuse)
{
    if (m.zero_copy) return GMLE_OK;
    for (const TableLaunch &L : plan.launches) {
        TableBufs &b = m.tables[L.kind];
        // the device table is rewritten after the last launch that read it
        CK(cudaStreamWaitEvent(s, b.used, 0), "cudaStreamWaitEvent");
        CK(cudaMemcpyAsync(b.d_base, b.h_base, kTableHeader + sizeof(KernelArgs) * L.groups,
                           cudaMemcpyHostToDevice, s), "H2D group table");
        CK(cudaMemcpyAsync(b.d_base + b.tiles_off(), b.h_base + b.tiles_off(),
                           sizeof(int64_t) * L.tiles, cudaMemcpyHostToDevice, s), "H2D tile map");
        if (record_reuse) CK(cudaEventRecord(b.reuse, s), "cudaEventRecord");
    }
    return GMLE_OK;
}

gmle_status enqueue_table_launch(gmle_ctx *ctx, MixedSet &m, const TableLaunch &L, cudaStream_t q)
{
    TableBufs &b = m.tables[L.kind];
    const char *base = m.zero_copy ? b.h_base : b.d_base;
    gmle::TileTable t;
    t.header = reinterpret_cast<const int64_t *>(base);
    t.groups = reinterpret_cast<const KernelArgs *>(base + kTableHeader);
    t.tiles = reinterpret_cast<const int64_t *>(base + b.tiles_off());
    t.tile0 = nullptr;
    t.counter = L.persistent ? b.d_counter : nullptr;
    KernelArgs a;
    std::memset(&a, 0, sizeof a);
    a.tpr = L.shape.tpr;
    if (L.persistent)
        CK(cudaMemsetAsync(b.d_counter, 0, sizeof(unsigned long long), q), "reset tile counter");
    ctx->launches++;
    CK(gmle::launch_fit(L.model, L.box, L.scmos, a, t, L.shape, q), "table launch");
    if (!m.zero_copy) CK(cudaEventRecord(b.used, q), "cudaEventRecord");
    return GMLE_OK;
}

int plan_stream(int index, bool holds_tmem, int nf)
{
    // Persistent launches whose kernel holds tensor memory run in sequence on
    // fork 0: a persistent CTA keeps its columns until its launch runs out of
    // tiles, so a concurrent one's CTAs would wait in tcgen05.alloc on the
    // same SMs.  The others spread over the remaining forks.
    if (nf <= 1 || holds_tmem) return 0;
    return 1 + index % (nf - 1);
}

gmle_status enqueue_plan(gmle_ctx *ctx, MixedSet &m, const MixedPlan &plan, cudaStream_t s)
{
    // The launches of a plan (plain launches of large groups, table launches
    // of the rest) run concurrently on the fork streams, joined back into s,
    // so that each launch's last, partly filled wave overlaps the others.
    const int np = (int)plan.plain.size(), nl = (int)plan.launches.size();
    const int units = np + nl;
    const bool fork = units > 1;
    const int nf = fork ? std::min(units, kForks) : 0;
    if (fork) {
        CK(cudaEventRecord(m.ev_fork, s), "cudaEventRecord");
        for (int f = 0; f < nf; f++)
            CK(cudaStreamWaitEvent(m.fork[f], m.ev_fork, 0), "cudaStreamWaitEvent");
    }
    for (int u = 0; u < np; u++) {
        const gmle_group &G = plan.plain[u];
        const Tuning t = pick_tuning(ctx, &G.desc, G.n);
        KernelArgs a = make_args(ctx, &G.desc, G.data, G.x_corners, G.y_corners, G.n, G.params,
                                 G.crlb, G.llr, G.flags, t.tpr);
        // plain launches are not persistent (a CTA frees its tensor memory
        // after one tile), so they overlap freely
        CK(launch(ctx, &G.desc, a, t.rois_per_block, fork ? m.fork[u % nf] : s),
           "fit kernel launch");
    }
    for (int l = 0; l < nl; l++) {
        const TableLaunch &L = plan.launches[l];
        const bool tm = L.persistent && holds_tmem(L.scmos, L.shape.tpr);
        const gmle_status st = enqueue_table_launch(
            ctx, m, L, fork ? m.fork[plan_stream(np + l, tm, nf)] : s);
        if (st != GMLE_OK) return st;
    }
    for (int f = 0; f < nf; f++) {
        CK(cudaEventRecord(m.ev_join[f], m.fork[f]), "cudaEventRecord");
        CK(cudaStreamWaitEvent(s, m.ev_join[f], 0), "cudaStreamWaitEvent");
    }
    return GMLE_OK;
}

}  // namespace gmle_rt

extern "C" gmle_status gmle_fit_mixed_device(gmle_ctx *ctx, const gmle_group *groups,
                                             int32_t ngroups, void *stream)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ngroups < 0 || (ngroups > 0 && !groups))
        return fail(ctx, GMLE_INVALID_ARG, "groups array is required");
    cudaSetDevice(ctx->device);
    gmle_status st = init_mixed_set(ctx, ctx->mixed);
    if (st != GMLE_OK) return st;
    MixedPlan plan;
    st = plan_mixed(ctx, groups, ngroups, ctx->mixed, plan, PlanOptions());
    if (st != GMLE_OK) return st;
    st = upload_plan(ctx, ctx->mixed, plan, (cudaStream_t)stream, true);
    if (st != GMLE_OK) return st;
    return enqueue_plan(ctx, ctx->mixed, plan, (cudaStream_t)stream);
}
