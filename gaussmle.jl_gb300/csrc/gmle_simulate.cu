// gmle_simulate.cu - synthetic ROIs on the device (gmle_simulate_device).
//
// The reference simulator (src/simulator.jl:228-307, `_generate_single_roi!`)
// draws, per pixel (i, j) of a ROI, Poisson(mu) photo-electrons with
// mu = bg + N psf_x(j) psf_y(i) (`_evaluate_psf_pixel`, src/simulator.jl:
// 312-346); an sCMOS camera adds Normal(0, readnoise) and converts to ADU,
// total / gain + offset.  This kernel makes the same stacks at GPU rates, as
// benchmark input and as a check of the noise model against the fits.  Its
// random streams are its own (the reference's Julia RNG and Poisson sampler
// cannot be reproduced):
//
// * Philox4x32-10 (Salmon, Moraes, Dror and Shaw, "Parallel random numbers:
//   as easy as 1, 2, 3", SC 2011): key = the 64-bit seed, counter = (pixel
//   index, ROI index low word, high word, block), so a pixel's draws depend
//   only on (seed, ROI, pixel), whatever the launch shape; a 32-bit word w
//   gives the uniform (w + 0.5) / 2^32 in double, or ((w >> 8) + 0.5) / 2^24
//   in float (exact in both);
// * Poisson(lam): lam < 10 by inversion in float (sequential search of the
//   CDF from expf(-lam)), lam >= 10 by Hormann's transformed rejection with
//   squeeze (PTRS, "The transformed rejection method for generating Poisson
//   random variables", 1993), in float but for the exact acceptance test at
//   lam >= 64, in double; lam <= 0 gives 0 as in the reference;
// * read noise by Box-Muller in float from its own counter block;
// * mu in float from erf-integrated 1-D Gaussians (src/gausslib/
//   baselibrary.jl:8-14; astigmatic widths sigma0 sqrt(alpha(z -+ gamma)),
//   baselibrary.jl:75-83), the camera arithmetic in float in the
//   reference's order, every operation rounded on its own (no contraction).
//
// Maps are indexed like the fitting kernel, row = y (the reference simulator
// indexes its maps transposed, src/simulator.jl:292-304).  Layout: ROI k's
// pixel (i, j) at (i-1) + box (j-1) + box^2 k, true parameters (P, n)
// column-major in the fitted parameter order.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "gmle_internal.h"

namespace {

constexpr int kSimThreads = 256;
constexpr int kSimPixels = 2048;  // output pixels per block (whole ROIs)
constexpr int kSimMaxRois = 64;   // ROIs per block (axis tables in shared memory)
constexpr int kSimMaxBox = 32;
constexpr uint32_t kNoiseBlock = 0xFFFF;  // counter block of the read-noise draw

struct Words {
    uint32_t w[4];
};

// Philox4x32-10 of counter c with key (k0, k1).
__device__ __forceinline__ Words philox4x32_10(Words c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.w[0]), lo0 = 0xD2511F53u * c.w[0];
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.w[2]), lo1 = 0xCD9E8D57u * c.w[2];
        c = Words{{hi1 ^ c.w[1] ^ k0, lo1, hi0 ^ c.w[3] ^ k1, lo0}};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

__device__ __forceinline__ double to_uniform(uint32_t w) { return ((double)w + 0.5) * 0x1p-32; }
__device__ __forceinline__ float to_uniform_f(uint32_t w)
{
    return ((float)(w >> 8) + 0.5f) * 0x1p-24f;
}

// The uniforms of one pixel, from blocks 0, 1, 2, ... of its counter.
struct PixelStream {
    uint32_t k0, k1, p, rlo, rhi, block;
    Words words;
    int used;
    __device__ uint32_t word()
    {
        if (used == 4) {
            words = philox4x32_10(Words{{p, rlo, rhi, block}}, k0, k1);
            block++;
            used = 0;
        }
        return words.w[used++];
    }
    __device__ double uniform() { return to_uniform(word()); }
    __device__ float uniform_f() { return to_uniform_f(word()); }
};

// ln k! for integer k >= 0: a table below 10, else the Stirling series
// (k + 1/2) ln(k + 1) - (k + 1) + ln(2 pi)/2 + 1/(12 (k+1)) - 1/(360 (k+1)^3)
// for ln Gamma(k + 1), good to 1e-10 there.  Every operation rounded on its
// own, in float or in double.
__device__ __forceinline__ double log_factorial_table(int i)
{
    return i <= 1 ? 0.0 : i == 2 ? 0.6931471805599453 : i == 3 ? 1.791759469228055
         : i == 4 ? 3.1780538303479458 : i == 5 ? 4.787491742782046 : i == 6 ? 6.579251212010101
         : i == 7 ? 8.525161361065415 : i == 8 ? 10.60460290274525 : 12.801827480081469;
}
__device__ __forceinline__ float log_factorial_f(float k)
{
    if (k < 10.f) return (float)log_factorial_table((int)k);
    const float x = __fadd_rn(k, 1.0f), rx = __fdiv_rn(1.0f, x);
    const float corr = __fmul_rn(rx, __fadd_rn(0.0833333333f, -__fmul_rn(__fmul_rn(rx, rx), 0.00277777778f)));
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(__fadd_rn(k, 0.5f), logf(x)), -x), 0.918938533f), corr);
}
__device__ __forceinline__ double log_factorial_d(double k)
{
    if (k < 10.0) return log_factorial_table((int)k);
    const double x = __dadd_rn(k, 1.0), rx = __ddiv_rn(1.0, x);
    const double corr = __dmul_rn(rx, __dadd_rn(0.083333333333333333,
                                                -__dmul_rn(__dmul_rn(rx, rx), 0.0027777777777777778)));
    return __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(__dadd_rn(k, 0.5), log(x)), -x), 0.9189385332046728),
                     corr);
}

__device__ int64_t poisson_draw(double lam, PixelStream &s)
{
    if (!(lam > 0.0)) return 0;
    if (lam < 10.0) {
        const float lf = (float)lam;
        const float u = s.uniform_f();
        float p = expf(-lf), f = p;
        int64_t k = 0;
        while (u > f && k < 1000) {
            k++;
            p = __fmul_rn(p, __fdiv_rn(lf, (float)k));
            f = __fadd_rn(f, p);
        }
        return k;
    }
    const float lf = (float)lam;
    const float slam = __fsqrt_rn(lf);
    const float b = __fadd_rn(0.931f, __fmul_rn(2.53f, slam));
    const float a = __fadd_rn(-0.059f, __fmul_rn(0.02483f, b));
    const float invalpha = __fadd_rn(1.1239f, __fdiv_rn(1.1328f, __fadd_rn(b, -3.4f)));
    const float vr = __fadd_rn(0.9277f, -__fdiv_rn(3.6224f, __fadd_rn(b, -2.0f)));
    const double ld = (double)lf, loglam = lf < 64.f ? 0.0 : log(ld);
    const float loglamf = logf(lf);
    for (int it = 0; it < 10000; it++) {
        const float u = __fadd_rn(s.uniform_f(), -0.5f);
        const float v = s.uniform_f();
        const float us = __fadd_rn(0.5f, -fabsf(u));
        const float k = floorf(__fadd_rn(__fadd_rn(__fmul_rn(__fadd_rn(__fdiv_rn(__fmul_rn(2.0f, a), us),
                                                                       b), u), lf), 0.43f));
        if (us >= 0.07f && v <= vr) return (int64_t)k;
        if (k < 0.f || (us < 0.013f && v > us)) continue;
        // the exact test: log(v invalpha / (a / us^2 + b)) <= log p(k); in
        // float while its terms stay small, else in double
        if (lf < 64.f) {
            const float lhs = __fadd_rn(__fadd_rn(logf(v), logf(invalpha)),
                                        -logf(__fadd_rn(__fdiv_rn(a, __fmul_rn(us, us)), b)));
            const float rhs = __fadd_rn(__fadd_rn(-lf, __fmul_rn(k, loglamf)), -log_factorial_f(k));
            if (lhs <= rhs) return (int64_t)k;
        } else {
            const double usd = us, kd = k;
            const double lhs = __dadd_rn(__dadd_rn(log((double)v), log((double)invalpha)),
                                         -log(__dadd_rn(__ddiv_rn((double)a, __dmul_rn(usd, usd)),
                                                        (double)b)));
            const double rhs = __dadd_rn(__dadd_rn(-ld, __dmul_rn(kd, loglam)), -log_factorial_d(kd));
            if (lhs <= rhs) return (int64_t)k;
        }
    }
    return (int64_t)floorf(lf);
}

// erf-integrated 1-D Gaussian of pixel t (1-based) around c with width s.
__device__ __forceinline__ float integral_1d(int t, float c, float s)
{
    const float k = __fdiv_rn(1.0f, __fmul_rn(1.41421356f, s));
    const float d = __fadd_rn((float)t, -c);
    return __fmul_rn(0.5f, __fadd_rn(erff(__fmul_rn(__fadd_rn(d, 0.5f), k)),
                                     -erff(__fmul_rn(__fadd_rn(d, -0.5f), k))));
}

__device__ __forceinline__ float astig_width(float s0, float u, float a, float b)
{
    const float u2 = __fmul_rn(u, u);
    return __fmul_rn(s0, __fsqrt_rn(__fadd_rn(__fadd_rn(__fadd_rn(1.0f, u2), __fmul_rn(a, __fmul_rn(u2, u))),
                                              __fmul_rn(b, __fmul_rn(u2, u2)))));
}

struct SimArgs {
    int model, box, camera, P;
    float psf[8];
    const float *truth;
    const int32_t *xc, *yc;
    int64_t n;
    uint32_t k0, k1;
    const float *var, *gain, *offset;
    int32_t ny, nx;
    float *out;
    unsigned long long *bad;
};

__global__ void __launch_bounds__(kSimThreads) simulate_kernel(const SimArgs a, int rois_per_block)
{
    __shared__ float s_ax[kSimMaxRois][2][kSimMaxBox];  // [roi][x, y][pixel]
    __shared__ float s_n[kSimMaxRois], s_bg[kSimMaxRois];
    __shared__ long long s_base[kSimMaxRois];  // map offset of the ROI's first pixel; -1: bad
    const int box = a.box, b2 = box * box;
    const int64_t k0 = (int64_t)blockIdx.x * rois_per_block;
    const int64_t left = a.n - k0;
    const int nk = left < rois_per_block ? (int)left : rois_per_block;
    if (nk <= 0) return;
    // per ROI: photons, background and (sCMOS) the map offset
    for (int q = threadIdx.x; q < nk; q += blockDim.x) {
        const float *th = a.truth + (int64_t)a.P * (k0 + q);
        const int in = a.model == 3 ? 3 : 2, ib = a.model == 3 ? 4 : 3;
        s_n[q] = th[in];
        s_bg[q] = th[ib];
        long long base = 0;
        if (a.camera != GMLE_CAMERA_POISSON) {
            const int32_t x0 = a.xc[k0 + q], y0 = a.yc[k0 + q];
            const bool ok = x0 >= 1 && y0 >= 1 && (int64_t)x0 + box - 1 <= a.nx &&
                            (int64_t)y0 + box - 1 <= a.ny;
            if (!ok) atomicAdd(a.bad, 1ull);
            base = ok ? (long long)(y0 - 1) + (long long)a.ny * (x0 - 1) : -1;
        }
        s_base[q] = base;
    }
    // axis tables: entry (roi, axis, pixel index)
    for (int e = threadIdx.x; e < nk * 2 * box; e += blockDim.x) {
        const int q = e / (2 * box), r = e - q * 2 * box, ax = r / box, t = r - ax * box;
        const float *th = a.truth + (int64_t)a.P * (k0 + q);
        const float c = ax == 0 ? th[0] : th[1];
        float s;
        if (a.model == 0) {
            s = a.psf[0];
        } else if (a.model == 1) {
            s = th[4];
        } else if (a.model == 2) {
            s = ax == 0 ? th[4] : th[5];
        } else {
            const float z = th[2], gam = a.psf[6], d = a.psf[7];
            s = ax == 0 ? astig_width(a.psf[0], __fdiv_rn(__fadd_rn(z, -gam), d), a.psf[2], a.psf[4])
                        : astig_width(a.psf[1], __fdiv_rn(__fadd_rn(z, gam), d), a.psf[3], a.psf[5]);
        }
        s_ax[q][ax][t] = integral_1d(t + 1, c, s);
    }
    __syncthreads();
    const float qnan = __int_as_float(0x7fc00000);
    for (int e = threadIdx.x; e < nk * b2; e += blockDim.x) {
        const int q = e / b2, p = e - q * b2, j = p / box, i = p - j * box;
        const int64_t k = k0 + q;
        float *dst = a.out + k * b2 + p;
        const long long base = s_base[q];
        if (base < 0) {
            *dst = qnan;
            continue;
        }
        // mu = bg + N (psf_y[i] psf_x[j])
        const float mu = __fadd_rn(s_bg[q], __fmul_rn(s_n[q], __fmul_rn(s_ax[q][1][i], s_ax[q][0][j])));
        PixelStream st{a.k0, a.k1, (uint32_t)p, (uint32_t)k, (uint32_t)((uint64_t)k >> 32), 0u,
                       Words{}, 4};
        const int64_t cnt = poisson_draw(mu, st);
        if (a.camera == GMLE_CAMERA_POISSON) {
            *dst = (float)cnt;
            continue;
        }
        const long long m = base + i + (long long)a.ny * j;
        const Words w = philox4x32_10(Words{{(uint32_t)p, (uint32_t)k, (uint32_t)((uint64_t)k >> 32),
                                             kNoiseBlock}}, a.k0, a.k1);
        const float u1 = to_uniform_f(w.w[0]), u2 = to_uniform_f(w.w[1]);
        const float z = __fmul_rn(__fsqrt_rn(__fmul_rn(-2.0f, logf(u1))),
                                  cosf(__fmul_rn(6.28318530717958648f, u2)));
        const float tot = __fadd_rn((float)cnt, __fmul_rn(z, __fsqrt_rn(a.var[m])));
        *dst = a.camera == GMLE_CAMERA_SCMOS ? tot
                                             : __fadd_rn(__fdiv_rn(tot, a.gain[m]), a.offset[m]);
    }
}

}  // namespace

extern "C" gmle_status gmle_simulate_device(gmle_ctx *ctx, const gmle_fit_desc *d,
                                            const float *d_truth, const int32_t *d_x_corners,
                                            const int32_t *d_y_corners, int64_t n, uint64_t seed,
                                            float *d_rois, void *stream)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!d) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "desc is NULL");
    if (d->model < 0 || d->model > 3)
        return gmle_rt::fail(ctx, GMLE_UNSUPPORTED_MODEL, "unknown model id %d", d->model);
    if (d->box < 1 || d->box > kSimMaxBox)
        return gmle_rt::fail(ctx, GMLE_UNSUPPORTED_BOX, "box %d outside 1..%d", d->box, kSimMaxBox);
    if (d->camera < 0 || d->camera > 2)
        return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "unknown camera id %d", d->camera);
    if (n < 0) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "n < 0");
    if (n == 0) return GMLE_OK;
    if (!d_truth || !d_rois) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "truth and output are required");
    if (d->camera != GMLE_CAMERA_POISSON) {
        if (!d_x_corners || !d_y_corners)
            return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "sCMOS ROIs need their corners");
        if (!ctx->d_var) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "sCMOS ROIs without calibration maps");
        if (d->camera == GMLE_CAMERA_SCMOS_ADU && (!ctx->d_gain || !ctx->d_offset))
            return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "ADU ROIs need gain and offset maps");
    }
    SimArgs a{};
    a.model = d->model;
    a.box = d->box;
    a.camera = d->camera;
    a.P = gmle_rt::nparams(d->model);
    std::copy(d->psf, d->psf + 8, a.psf);
    a.truth = d_truth;
    a.xc = d_x_corners;
    a.yc = d_y_corners;
    a.n = n;
    a.k0 = (uint32_t)seed;
    a.k1 = (uint32_t)(seed >> 32);
    a.var = ctx->d_var;
    a.gain = ctx->d_gain;
    a.offset = ctx->d_offset;
    a.ny = ctx->ny;
    a.nx = ctx->nx;
    a.out = d_rois;
    a.bad = ctx->d_bad;
    cudaSetDevice(ctx->device);
    const int rpb = std::min(kSimMaxRois, std::max(1, kSimPixels / (d->box * d->box)));
    const int64_t blocks = (n + rpb - 1) / rpb;
    if (blocks > 0x7fffffffLL) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "too many ROIs");
    ctx->launches++;
    simulate_kernel<<<(unsigned)blocks, kSimThreads, 0, static_cast<cudaStream_t>(stream)>>>(a, rpb);
    GMLE_CK(cudaGetLastError(), "ROI generator launch");
    return GMLE_OK;
}
