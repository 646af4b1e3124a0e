/*
 * gaussmle_gb300.h - C ABI of libgaussmle_sm100a.so, the GB300 (sm_103a)
 * implementation of GaussMLE.jl's batched per-ROI Gaussian MLE fit.
 *
 * The library replaces the GPU branches of GaussMLE.fit
 * (src/interface.jl:217-263 for fit(Array), :334-370 for fit(ROIBatch{IdealCamera}),
 * :421-457 for fit(ROIBatch{SCMOSCamera})): every per-batch KernelAbstractions
 * allocate/copyto!/launch/synchronize/copy-back cycle becomes one call here.
 * Everything before those branches (input validation, to_pixel_units, corner
 * vectors) and after them (p-values, create_localization_result, to_smld)
 * stays on the caller's side, so the caller still builds the same emitters.
 *
 * Conventions (the reference's, src/unified_kernel.jl:285-297):
 *  - data is Float32 (box, box, n) column-major: pixel (i = row = y,
 *    j = column = x) of ROI k is data[(i-1) + box*(j-1) + box*box*k];
 *  - camera maps are Float32 (ny, nx) column-major, map[row = y, col = x];
 *  - corners are 1-based Int32 (Julia): ROI pixel (i, j) of ROI k lies on
 *    camera pixel (row = y_corners[k] + i - 1, col = x_corners[k] + j - 1);
 *  - outputs: params[k + P*roi] and crlb[k + P*roi] (Julia's results[k, idx],
 *    uncertainties[k, idx]), llr[roi], flags[roi].
 *  - parameter order per model: XYNB [x, y, N, bg]; XYNBS [x, y, N, bg, s];
 *    XYNBSXSY [x, y, N, bg, sx, sy]; AstigmaticXYZNB [x, y, z, N, bg]
 *    (src/psf_models.jl:20-24, 48-53, 74-80, 107-112). x, y are ROI pixels
 *    (pixel centres at 1..box), sigmas in pixels, z in the units of gamma and d.
 *
 * Errors: every call returns a gmle_status; no exception or exit crosses the
 * ABI; gmle_last_error() gives the message of the context's last failure.
 * A per-ROI numerical failure is not an error: the ROI's CRLB is Inf and its
 * GMLE_FLAG_CONVERGED bit is clear, as in src/unified_kernel.jl:424-430.
 * There is no CPU fallback: without a usable GB300, gmle_create fails.
 */
#ifndef GAUSSMLE_GB300_H
#define GAUSSMLE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GMLE_ABI_VERSION 1

typedef enum {
    GMLE_OK = 0,
    GMLE_INVALID_ARG = 1,
    GMLE_UNSUPPORTED_MODEL = 2,
    GMLE_UNSUPPORTED_BOX = 3,
    GMLE_OUT_OF_MEMORY = 4,
    GMLE_ADMISSION_REJECTED = 5,
    GMLE_CUDA_ERROR = 6,
    GMLE_TIMEOUT = 7,
    GMLE_NO_DEVICE = 8,
    GMLE_NOT_READY = 9
} gmle_status;

/* PSF models, src/psf_models.jl:39-154 */
typedef enum {
    GMLE_MODEL_XYNB = 0,     /* GaussianXYNB: fixed sigma, P = 4 */
    GMLE_MODEL_XYNBS = 1,    /* GaussianXYNBS: fitted sigma, P = 5 */
    GMLE_MODEL_XYNBSXSY = 2, /* GaussianXYNBSXSY: fitted sigma_x, sigma_y, P = 6 */
    GMLE_MODEL_ASTIG = 3     /* AstigmaticXYZNB: P = 5 */
} gmle_model;

/* Camera noise models, src/camera_models.jl:19-42 */
typedef enum {
    GMLE_CAMERA_POISSON = 0,   /* IdealCamera: Poisson likelihood */
    GMLE_CAMERA_SCMOS = 1,     /* SCMOSCamera: data already in e-, variance map resident */
    GMLE_CAMERA_SCMOS_ADU = 2  /* SCMOSCamera: data in ADU; e- = (ADU - offset) * gain
                                  applied on the device (src/camera_models.jl:110-113) */
} gmle_camera;

/* Iteration method of a fit. */
typedef enum {
    GMLE_METHOD_NEWTON = 0,    /* the reference's per-parameter Newton step with its diagonal
                                  Hessian (src/unified_kernel.jl:330-350); the default */
    GMLE_METHOD_FISHER_LM = 1  /* no reference counterpart: full-Hessian steps, (F + lambda
                                  diag F) step = gradient with the expected information F
                                  (Fisher scoring) and Levenberg-Marquardt damping; a step
                                  that lowers the log-likelihood is rejected (lambda x 10,
                                  step halved).  Same clamps, same final pass and CRLB.
                                  gmle_fit and gmle_fit_device only, one thread per ROI */
} gmle_method;

/* Per-ROI output flag bits */
#define GMLE_FLAG_CONVERGED 1u /* isfinite(CRLB_x): test/local_performance_benchmark.jl:291-293 */
#define GMLE_FLAG_CHOLESKY 2u  /* Fisher inverse via Cholesky (src/unified_kernel.jl:412) */
#define GMLE_FLAG_LU 4u        /* LU fallback (src/unified_kernel.jl:419) */
#define GMLE_FLAG_SINGULAR 8u  /* both failed: CRLB = Inf (src/unified_kernel.jl:424-430) */

/*
 * Fit descriptor: the non-array arguments of unified_gaussian_mle_kernel!
 * (src/unified_kernel.jl:286-297).
 *  psf[]: model constants in PIXEL units (after to_pixel_units,
 *         src/psf_models.jl:311-331): XYNB psf[0] = sigma; XYNBS, XYNBSXSY
 *         unused; astigmatic psf = {sx0, sy0, Ax, Ay, Bx, By, gamma, d}.
 *  lower/upper/max_step: ParameterConstraints (src/constraints.jl:5-9), first
 *         P entries used.
 */
typedef struct {
    int32_t model;      /* gmle_model */
    int32_t box;        /* ROI edge length 3..64 (gmle_fit, gmle_fit_device); 3..16 in
                           mixed batches, serving and the no-allocation entry point */
    int32_t iterations; /* Newton iterations (reference default 20) */
    int32_t camera;     /* gmle_camera */
    float psf[8];
    float lower[6];
    float upper[6];
    float max_step[6];
    int32_t method;     /* gmle_method; 0 (zero-initialised) is the reference's */
} gmle_fit_desc;

typedef struct gmle_ctx gmle_ctx;

/* Library ABI version (GMLE_ABI_VERSION). */
int gmle_abi_version(void);

/*
 * Create a context on CUDA device `device_ordinal`: device selection replaces
 * src/devices.jl:5-35 without its CPU fallback (returns GMLE_NO_DEVICE).
 */
gmle_status gmle_create(gmle_ctx **out, int device_ordinal);
void gmle_destroy(gmle_ctx *ctx);
const char *gmle_last_error(const gmle_ctx *ctx);

/*
 * Upload camera calibration maps once; they stay resident on the device and
 * are used by every sCMOS fit of this context.  variance = readnoise^2 in e-^2
 * (extract_variance_map, src/interface.jl:43-55); gain (e-/ADU) and offset
 * (ADU) may be NULL when only GMLE_CAMERA_SCMOS fits are made.  Maps are
 * (ny, nx) column-major.  Replaces the per-batch map upload of
 * src/interface.jl:431-432.
 */
gmle_status gmle_set_calibration(gmle_ctx *ctx, const float *variance, const float *gain,
                                 const float *offset, int32_t ny, int32_t nx);

/*
 * Synchronous fit of n ROIs from HOST memory into HOST memory: the whole GPU
 * branch of fit (src/interface.jl:220-262 and its ROIBatch twins).  Pinned
 * caller buffers are copied by DMA directly; pageable ones are staged through
 * the context's pinned buffers.  Transfers of one chunk overlap the fit of
 * the previous one.  x_corners / y_corners may be NULL for Poisson fits;
 * flags may be NULL.
 */
gmle_status gmle_fit(gmle_ctx *ctx, const gmle_fit_desc *desc, const float *data,
                     const int32_t *x_corners, const int32_t *y_corners, int64_t n,
                     float *params, float *crlb, float *llr, uint8_t *flags);

/*
 * Asynchronous fit of n ROIs already resident in DEVICE memory (for callers
 * that hold device arrays, e.g. a CuArray): enqueues the fit kernel on
 * `stream` (a cudaStream_t, used as given: NULL is the legacy default
 * stream, as everywhere in CUDA) and returns.  All
 * pointers are device pointers; flags may be NULL.  Corners outside the
 * calibration map are reported through gmle_fit_device_errors().
 */
gmle_status gmle_fit_device(gmle_ctx *ctx, const gmle_fit_desc *desc, const float *d_data,
                            const int32_t *d_x_corners, const int32_t *d_y_corners, int64_t n,
                            float *d_params, float *d_crlb, float *d_llr, uint8_t *d_flags,
                            void *stream);

/* Number of ROIs rejected by device-side corner checks since the last call
 * (synchronises the context's stream). */
gmle_status gmle_fit_device_errors(gmle_ctx *ctx, int64_t *count);

/*
 * Kernel launch shape used for a (model, box, camera): threads per ROI and
 * ROIs per block, as picked by the autotuner (or set by gmle_set_tuning;
 * setting (0, 0) forgets the entry and restores the size-based default).
 * Threads per ROI: 1, 2, 4, or 8 (2 and 8 for odd boxes 5..15 only); one thread per
 * ROI allows at most 128 ROIs per block, several lanes 256 threads per block.
 * Boxes 3..16; larger boxes run in one fixed shape.
 */
gmle_status gmle_get_tuning(gmle_ctx *ctx, int32_t model, int32_t box, int32_t camera,
                            int32_t *threads_per_roi, int32_t *rois_per_block);
gmle_status gmle_set_tuning(gmle_ctx *ctx, int32_t model, int32_t box, int32_t camera,
                            int32_t threads_per_roi, int32_t rois_per_block);

/*
 * Autotuner: times every candidate launch shape (threads per ROI 1, 2, 4, 8;
 * 32..256 threads per block, within 227 KiB of shared memory) of the fit
 * kernel for `desc` on a device-resident batch, keeps the fastest for
 * (model, box, camera family) in the context and returns it with its time
 * per launch.  The output buffers are overwritten.  No reference counterpart:
 * KernelAbstractions picks the reference's workgroup size.
 */
gmle_status gmle_autotune(gmle_ctx *ctx, const gmle_fit_desc *desc, const float *d_data,
                          const int32_t *d_x_corners, const int32_t *d_y_corners, int64_t n,
                          float *d_params, float *d_crlb, float *d_llr, uint8_t *d_flags,
                          int32_t *threads_per_roi, int32_t *rois_per_block, float *ms_per_fit);

/*
 * Cut n box x box ROIs out of device-resident camera frames into the
 * (box, box, n) stack that gmle_fit_device takes.  In the reference pipeline a
 * box finder does this on the host and hands GaussMLE a ROIBatch of ROI stack,
 * corners and frame indices (examples/full_pipeline_boxer.jl:72-103).
 * frames: Float32 (ny, nx, nframes) column-major; frame indices and corners:
 * 1-based Int32, ROI pixel (i, j) of ROI k = frame pixel
 * (y_corners[k] + i - 1, x_corners[k] + j - 1, frame_idx[k]).  All pointers are
 * device pointers; the copy is enqueued on `stream`.  An ROI whose frame or box
 * lies outside the stack is filled with NaN and counted by
 * gmle_fit_device_errors (synchronise `stream` before asking).
 */
gmle_status gmle_cut_rois_device(gmle_ctx *ctx, const float *d_frames, int32_t ny, int32_t nx,
                                 int64_t nframes, const int32_t *d_frame_idx,
                                 const int32_t *d_x_corners, const int32_t *d_y_corners,
                                 int64_t n, int32_t box, float *d_rois, void *stream);

/*
 * Synthetic ROIs on the device, in the (box, box, n) layout gmle_fit_device
 * takes.  Replaces the reference simulator's per-ROI loop
 * (src/simulator.jl:228-307): pixel (i, j) of ROI k has the expectation
 * mu = bg + N psf_x(j) psf_y(i) of its true parameters d_truth[P k ...]
 * ((P, n) column-major, the fitted parameter order of d->model; d->psf as for
 * fitting; d->iterations and the constraints are not used), then
 *   GMLE_CAMERA_POISSON:   Poisson(mu);
 *   GMLE_CAMERA_SCMOS:     Poisson(mu) + Normal(0, variance) in electrons;
 *   GMLE_CAMERA_SCMOS_ADU: (Poisson(mu) + Normal(0, variance)) / gain + offset,
 * with the context's calibration maps at the ROI's 1-based corners (row = y;
 * corners may be NULL for Poisson).  Draws come from a counter-based
 * Philox4x32-10 stream keyed by `seed`: pixel p of ROI k depends only on
 * (seed, k, p).  Box sizes 1..32.  An sCMOS ROI whose box lies outside the
 * maps is filled with NaN and counted by gmle_fit_device_errors.  Device
 * pointers; enqueued on `stream`.  (No reference counterpart as an API: the
 * reference generates on the host, with its own random streams.)
 */
gmle_status gmle_simulate_device(gmle_ctx *ctx, const gmle_fit_desc *d, const float *d_truth,
                                 const int32_t *d_x_corners, const int32_t *d_y_corners,
                                 int64_t n, uint64_t seed, float *d_rois, void *stream);

/*
 * Goodness-of-fit p-values, computed on the GPU.  Replaces the host loop after
 * every fit (src/interface.jl:265-275, :459-468): chi2 = -2 llr in Float32 and
 * p = 1 - Float32(cdf(Chisq(df), chi2)), with df = box^2 - P for a fit of P
 * parameters.  cdf is evaluated in FP64 (the regularised incomplete gamma
 * function P(df/2, chi2/2)).  A NaN llr gives a NaN p-value; chi2 <= 0 gives 1.
 * gmle_pvalues takes host arrays and returns when the p-values are written;
 * gmle_pvalues_device takes device arrays and enqueues on `stream`.
 */
gmle_status gmle_pvalues(gmle_ctx *ctx, const float *llr, int64_t n, int32_t df, float *pvalues);
gmle_status gmle_pvalues_device(gmle_ctx *ctx, const float *d_llr, int64_t n, int32_t df,
                                float *d_pvalues, void *stream);

/*
 * Accuracy check of the fit kernels' own elementary functions (no reference
 * counterpart: the reference calls SpecialFunctions.erf and Base.exp).  For
 * each of the n device-resident arguments x[i], writes into d_out ((8, n),
 * row k at d_out + k n): 0 the fit's erf(x) (from exp(-x^2) at the same
 * edge), 1 the CUDA library's erff(x), 2 the fit's exp(-x^2 / 2), 3 expf of
 * the same, 4 the fit's 1/x, 5 the IEEE 1/x, 6 the fit's ln|x|, 7 logf(|x|).
 * Enqueued on `stream`.
 */
gmle_status gmle_math_selftest(const float *d_x, int64_t n, float *d_out, void *stream);

/* Number of fit-kernel launches this context has issued (for accounting). */
int64_t gmle_kernel_launches(const gmle_ctx *ctx);

/*
 * One homogeneous group of a mixed batch: its own fit descriptor and buffers.
 * Pointers are device pointers for gmle_fit_mixed_device and host pointers
 * for gmle_submit.
 */
typedef struct {
    gmle_fit_desc desc;
    const float *data;
    const int32_t *x_corners;
    const int32_t *y_corners;
    int64_t n;
    float *params;
    float *crlb;
    float *llr;
    uint8_t *flags;
} gmle_group;

/*
 * Fit a mixed batch (any mix of PSF models and box sizes 3..16) of
 * device-resident groups, enqueued on `stream` (used as given).  The groups of
 * each (camera family, model, box) present share one persistent,
 * work-stealing launch of that model's kernel; these launches run
 * concurrently.  A group of 65536 ROIs or more gets its own plain launch.  No
 * reference counterpart: the reference fits one (model, box) per fit() call
 * (src/interface.jl:177-291).
 */
gmle_status gmle_fit_mixed_device(gmle_ctx *ctx, const gmle_group *groups, int32_t ngroups,
                                  void *stream);

/*
 * gmle_fit_mixed_device for callers that cannot allocate device memory.  No
 * counterpart in the reference, which allocates its device arrays in every
 * fit() call (src/interface.jl:229-240, :341-349, :428-436).
 *
 * Who needs it: a host process whose device memory is owned by its own pool
 * allocator (CUDA.jl's memory pool, PyTorch's caching allocator) and that has
 * reserved most of the GPU for it, so an allocation by the library can fail or
 * break the pool's accounting.  Also code that must not call cudaMalloc
 * because it can synchronise the whole device and stall other streams.  Such
 * a caller brings its inputs and outputs in its own memory, and this call
 * adds nothing to the process's device memory.
 *
 * The call allocates nothing: no cudaMalloc, cudaFree, pinned memory, stream,
 * event or host heap, and it needs no context.  Its scratch is a static device
 * array of GMLE_NOALLOC_SCRATCH_BYTES (240,640 bytes).  The array holds the
 * persistent launches' group tables, their work-stealing tile counters and a
 * skipped-ROI counter.  It is reserved on each GPU that loads the library's
 * device code and stays there until the process exits.
 *
 * groups    Device pointers, as for gmle_fit_mixed_device.  At most
 *           GMLE_NOALLOC_MAX_GROUPS groups; a larger ngroups returns
 *           GMLE_INVALID_ARG and launches nothing.  Every group runs in the
 *           persistent launches, including groups of 65536 ROIs or more,
 *           with the size-based default launch shapes.
 * variance, gain, offset
 *           Device (ny, nx) column-major calibration maps.  NULL when the
 *           batch is Poisson-only; gain and offset are needed for
 *           GMLE_CAMERA_SCMOS_ADU.
 * stream    Must belong to the current device, which the call runs on; used
 *           as given.
 * err       May be NULL.  Receives a failure's message, up to err_len bytes.
 *
 * Set-up: the first call on a device looks up the scratch address
 * (cudaGetSymbolAddress); the first launch of each kernel on a device sets its
 * shared-memory limit.  Make that first call before any stream capture.
 *
 * Zeroing: the tile counters must be zero when each launch starts.  Every
 * call writes its tables into the scratch, ahead of its fit launches on
 * `stream`, by small kernels that carry the tables in their launch
 * parameters (one per 32 704 bytes: one for up to 95 groups); that write
 * sets the counters to zero.  The call does not wait for the stream.
 *
 * Overlap: all calls on a device share the one scratch.  Calls whose GPU work
 * overlaps race and give undefined results, e.g. calls on different streams
 * with no event ordering them.  Calls on one stream run in order.  On the
 * host, building a call's tables and enqueuing its launches hold one
 * process-wide lock, so calls from several threads (and devices) are
 * enqueued one after another; none of them waits for the GPU.
 */
#define GMLE_NOALLOC_MAX_GROUPS 1024
#define GMLE_NOALLOC_SCRATCH_BYTES (3072 + (8 + 224) * GMLE_NOALLOC_MAX_GROUPS)
gmle_status gmle_fit_mixed_device_noalloc(const gmle_group *groups, int32_t ngroups,
                                          const float *variance, const float *gain,
                                          const float *offset, int32_t ny, int32_t nx,
                                          void *stream, char *err, int32_t err_len);

/*
 * Serving loop (no reference counterpart: GaussMLE.fit is one blocking call
 * per batch, src/interface.jl:220-262).  A scheduler thread owned by the
 * context admits submitted requests into a device arena (admission by HBM
 * budget, FIFO), copies their ROIs in, and continuously batches every request
 * whose data has arrived into the next step: one table launch per (camera
 * family, model, box) present, with one block per tile of 32..128 ROIs.  Up
 * to max_inflight_steps steps run concurrently, and their blocks interleave
 * on the SMs, so requests that arrive while others are on the GPU start as
 * soon as SMs and memory free up.  Results land in the caller's host
 * buffers, which must stay valid until the request completes: outputs in
 * pinned (page-locked) memory are written there by the kernels, others are
 * copied back after the step.  ROI data and corner arrays in pinned memory
 * are read in place by the kernels (such a request needs no input copy and
 * can join the next step at once); others are copied in on one input stream,
 * in order.
 */
typedef struct {
    int64_t hbm_budget_bytes;   /* device arena; 0 = half of the free HBM at start */
    int32_t max_inflight_steps; /* concurrent steps; 0 = 4 (at most 8) */
    int64_t max_step_rois;      /* ROIs per step; 0 = 2^21 */
    int32_t max_pending;        /* queued requests before submit rejects; 0 = 1 << 16 */
    int32_t use_graphs;         /* 1: each launch is a replay of a captured CUDA graph of a
                                   persistent launch (fixed grid, blocks take tiles from a
                                   counter); 0 (default): direct launches, one block per tile */
} gmle_server_config;

typedef struct {
    int64_t submitted, completed, rejected, failed;
    int64_t rois_completed;
    int64_t steps;              /* kernel launches (graph replays) */
    double p50_latency_ms, p99_latency_ms, mean_latency_ms, max_latency_ms;
    double fits_per_s;          /* completed ROIs / (last completion - first submission) */
    int64_t hbm_budget_bytes, hbm_in_use_bytes, hbm_peak_bytes;
} gmle_server_stats;

gmle_status gmle_server_start(gmle_ctx *ctx, const gmle_server_config *config);
/* Finishes all admitted and queued work, then stops the scheduler. */
gmle_status gmle_server_stop(gmle_ctx *ctx);
/* Queue one request (host pointers, flags may be NULL).  GMLE_ADMISSION_REJECTED
 * when it can never fit the arena or the queue is full. */
gmle_status gmle_submit(gmle_ctx *ctx, const gmle_group *request, uint64_t *ticket);
/* gmle_submit of n requests in order, in one call: tickets[k] is request k's.
 * Stops at the first request that is not accepted and returns its status;
 * *submitted (may be NULL) is the number accepted before it.  The scheduler
 * is woken after the first request and every 16th, so that the first steps
 * start while later requests are still being queued. */
gmle_status gmle_submit_many(gmle_ctx *ctx, const gmle_group *requests, int32_t n,
                             uint64_t *tickets, int32_t *submitted);
/* GMLE_OK when the request is done (its outputs are written), GMLE_NOT_READY
 * while it runs, or the status it failed with.  A finished ticket is
 * forgotten once GMLE_OK (or its failure) has been returned. */
gmle_status gmle_poll(gmle_ctx *ctx, uint64_t ticket);
/* Like gmle_poll but blocks up to timeout_ns (< 0: forever); GMLE_TIMEOUT. */
gmle_status gmle_wait(gmle_ctx *ctx, uint64_t ticket, int64_t timeout_ns);
/* Counters and latency percentiles since start (or the last reset). */
gmle_status gmle_server_stats_get(gmle_ctx *ctx, gmle_server_stats *out, int32_t reset);

#ifdef __cplusplus
}
#endif

#endif /* GAUSSMLE_GB300_H */
