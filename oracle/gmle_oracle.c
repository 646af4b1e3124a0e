/*
 * CPU oracle for the batched per-ROI Gaussian MLE fit of GaussMLE.jl.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, on the CPU, the reference's
 * fit kernel `unified_gaussian_mle_kernel!` (src/unified_kernel.jl:285-434)
 * and everything it calls (src/psf_derivatives.jl, src/gausslib/baselibrary.jl,
 * src/camera_models.jl, src/constraints.jl).  Only the tests, the smoke check
 * and the CPU-baseline leg of the benchmark may load it, and only as the
 * checker; the product library (libgaussmle_sm100a.so) never calls it.
 *
 * Parity status: the reference is Julia and cannot run where this oracle is
 * built (no Julia toolchain), and the reference holds no golden vectors, so
 * value-level parity with the reference itself is UNPINNED.  The oracle is
 * pinned instead against (a) the astigmatic theoretical CRLB table published
 * in the reference's dev notes (dev/astig_theory/README.md:33-46, produced by
 * dev/astig_theory/compute_theoretical_crlb.jl), (b) the statistical
 * acceptance criteria of the reference's test-suite (std/CRLB ratios, biases,
 * the sCMOS variance-map x/y indexing test), re-expressed in tests/.
 *
 * Two builds of one body (gmle_oracle_body.h):
 *   *_f32  the reference's FP32 CPU path, op for op (compiled with
 *          -ffp-contract=off; Julia's x^4, x^5 and x^1.5f0 evaluate in
 *          Float64 and round once, reproduced below);
 *   *_f64  the same iteration in FP64: the error oracle.
 * erf comes from SpecialFunctions.jl 2.6.1 in the reference (openlibm erff,
 * not vendored); here it is the C library's erff/erf.  Both are within about
 * one ulp of the true function.
 *
 * Data layout (Julia column-major): pixel (i = row = y, j = column = x) of ROI
 * k is data[(i-1) + box*(j-1) + box*box*k]; camera maps are (ny, nx)
 * column-major; corners are 1-based.  Outputs: params[k + P*roi],
 * crlb[k + P*roi], llr[roi], flags[roi].
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_FLAG_CONVERGED 1u /* isfinite(CRLB_x): the reference benchmark's notion */
#define ORACLE_FLAG_CHOLESKY 2u
#define ORACLE_FLAG_LU 4u
#define ORACLE_FLAG_SINGULAR 8u

/* Same field layout and meaning as gmle_fit_desc in the product header; kept
 * separate so that the checker shares no code with what it checks. */
typedef struct {
    int32_t model;      /* 0 XYNB, 1 XYNBS, 2 XYNBSXSY, 3 AstigmaticXYZNB */
    int32_t box;        /* ROI edge length in pixels (3..ORACLE_MAX_BOX) */
    int32_t iterations; /* Newton iterations */
    int32_t camera;     /* 0 Poisson, 1 sCMOS (data in e-), 2 sCMOS (data in ADU) */
    float psf[8];
    float lower[6];
    float upper[6];
    float max_step[6];
    int32_t method;     /* 0 the reference's Newton step, 1 the library's full-Hessian option */
} oracle_desc;

/* largest ROI edge the oracle takes (the reference accepts any box >= 3,
 * src/interface.jl:22) */
#define ORACLE_MAX_BOX 64

static inline int oracle_nparams(int model)
{
    return model == 0 ? 4 : (model == 2 ? 6 : 5);
}

/* Julia's Float32 integer powers: Float32(power_by_squaring(Float64(x), n)) */
static inline float jl_pow4f(float x)
{
    double d = (double)x;
    double d2 = d * d;
    return (float)(d2 * d2);
}
static inline float jl_pow5f(float x)
{
    double d = (double)x;
    double d2 = d * d;
    return (float)(d * (d2 * d2));
}
/* Julia's Float32 ^ Float32 for a non-integer exponent: Float32(exp2(log2(x) * y)) in Float64 */
static inline float jl_pow15f(float x) { return (float)pow((double)x, 1.5); }

static inline double pow4d(double x) { double x2 = x * x; return x2 * x2; }
static inline double pow5d(double x) { double x2 = x * x; return x * (x2 * x2); }
static inline double pow15d(double x) { return pow(x, 1.5); }

/* ---- FP32 build ---- */
#define R float
#define FN(x) x##_f32
#define ERF erff
#define EXP expf
#define LOG logf
#define SQRT sqrtf
#define FABS fabsf
#define POW4(x) jl_pow4f(x)
#define POW5(x) jl_pow5f(x)
#define POW15(x) jl_pow15f(x)
#include "gmle_oracle_body.h"
#undef R
#undef FN
#undef ERF
#undef EXP
#undef LOG
#undef SQRT
#undef FABS
#undef POW4
#undef POW5
#undef POW15

/* ---- FP64 build ---- */
#define R double
#define FN(x) x##_f64
#define ERF erf
#define EXP exp
#define LOG log
#define SQRT sqrt
#define FABS fabs
#define POW4(x) pow4d(x)
#define POW5(x) pow5d(x)
#define POW15(x) pow15d(x)
#include "gmle_oracle_body.h"

/* ---- exported entry points ------------------------------------------------- */

static int check_desc(const oracle_desc *d)
{
    if (d->model < 0 || d->model > 3) return -1;
    if (d->box < 3 || d->box > ORACLE_MAX_BOX) return -2;
    if (d->iterations < 0) return -3;
    if (d->camera < 0 || d->camera > 2) return -4;
    if (d->method < 0 || d->method > 1) return -5;
    return 0;
}

int oracle_version(void) { return 1; }

/* FP32 restatement of the reference CPU path. nthreads <= 0: all cores. */
int oracle_fit_f32(const oracle_desc *d, const float *data, const int32_t *xc, const int32_t *yc,
                   int64_t n, const float *var, const float *gain, const float *offset,
                   int32_t ny, int32_t nx, float *params, float *crlb, float *llr,
                   uint8_t *flags, int nthreads)
{
    int rc = check_desc(d);
    if (rc) return rc;
    (void)nx;
    const int P = oracle_nparams(d->model);
    const int64_t b2 = (int64_t)d->box * d->box;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t r = 0; r < n; r++)
        fit_one_f32(d, data + b2 * r, xc ? xc[r] : 1, yc ? yc[r] : 1, var, gain, offset, ny,
                    params + P * r, crlb + P * r, llr + r, flags + r);
    return 0;
}

/* FP64 oracle of the same iteration (inputs are the same float arrays). */
int oracle_fit_f64(const oracle_desc *d, const float *data, const int32_t *xc, const int32_t *yc,
                   int64_t n, const float *var, const float *gain, const float *offset,
                   int32_t ny, int32_t nx, double *params, double *crlb, double *llr,
                   uint8_t *flags, int nthreads)
{
    int rc = check_desc(d);
    if (rc) return rc;
    (void)nx;
    const int P = oracle_nparams(d->model);
    const int64_t b2 = (int64_t)d->box * d->box;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t r = 0; r < n; r++)
        fit_one_f64(d, data + b2 * r, xc ? xc[r] : 1, yc ? yc[r] : 1, var, gain, offset, ny,
                    params + P * r, crlb + P * r, llr + r, flags + r);
    return 0;
}

/* The final pass (LLR, Fisher, CRLB) of n ROIs at given parameters theta
 * ((n, P) row-major doubles, e.g. another implementation's fitted values):
 * separates the error of a Fisher accumulation and inversion from that of the
 * Newton iterations that led to theta. */
int oracle_final_at_f32(const oracle_desc *d, const float *data, const int32_t *xc,
                        const int32_t *yc, int64_t n, const float *var, const float *gain,
                        const float *offset, int32_t ny, const double *theta, float *crlb,
                        float *llr, uint8_t *flags, int nthreads)
{
    int rc = check_desc(d);
    if (rc) return rc;
    const int P = oracle_nparams(d->model);
    const int64_t b2 = (int64_t)d->box * d->box;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t r = 0; r < n; r++)
        final_at_f32(d, data + b2 * r, xc ? xc[r] : 1, yc ? yc[r] : 1, var, gain, offset, ny,
                     theta + P * r, crlb + P * r, llr + r, flags + r);
    return 0;
}
int oracle_final_at_f64(const oracle_desc *d, const float *data, const int32_t *xc,
                        const int32_t *yc, int64_t n, const float *var, const float *gain,
                        const float *offset, int32_t ny, const double *theta, double *crlb,
                        double *llr, uint8_t *flags, int nthreads)
{
    int rc = check_desc(d);
    if (rc) return rc;
    const int P = oracle_nparams(d->model);
    const int64_t b2 = (int64_t)d->box * d->box;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
    for (int64_t r = 0; r < n; r++)
        final_at_f64(d, data + b2 * r, xc ? xc[r] : 1, yc ? yc[r] : 1, var, gain, offset, ny,
                     theta + P * r, crlb + P * r, llr + r, flags + r);
    return 0;
}

/* CRLB at fixed parameters (Poisson), FP32 and FP64; returns the flag bits. */
int oracle_crlb_at_f32(int model, int box, const float *psf, const double *theta, float *crlb)
{
    return crlb_at_theta_f32(model, box, psf, theta, crlb);
}
int oracle_crlb_at_f64(int model, int box, const float *psf, const double *theta, double *crlb)
{
    return crlb_at_theta_f64(model, box, psf, theta, crlb);
}

int oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
