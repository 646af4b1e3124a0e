// gmle_fit_kernel.cuh - the batched per-ROI Gaussian MLE fit for sm_103a.
//
// One kernel template per (PSF model, box size, camera family).  It computes
// what unified_gaussian_mle_kernel! computes (src/unified_kernel.jl:285-434):
// initialisation, `iterations` scalar Newton steps with clamped constraints,
// then the log-likelihood ratio, the Fisher matrix, its inverse and the CRLB.
//
// GB300 mapping (the reference runs one generic thread per ROI that re-reads
// global memory and recomputes 4 erf + 4 exp per pixel per iteration):
//  * A block owns `rois_per_block` consecutive ROIs, which are contiguous in
//    the Julia (box, box, n) layout; it stages them into shared memory with
//    coalesced 16-byte loads (plus the sCMOS variance tile gathered from the
//    resident calibration map, with the ADU->e- conversion fused in).
//  * `tpr` lanes (1..32, a power of two) fit one ROI; lane r owns pixel
//    columns j = r+1, r+1+tpr, ...  Per Newton iteration the model is
//    separable: per axis the erf/exp terms are evaluated once per pixel index
//    (box entries per axis instead of box^2 per pixel), the y-axis tables are
//    shared through shared memory and held in registers, and each pixel costs
//    a few FP32 FMAs.
//  * Gradient and diagonal Hessian are summed with warp shuffles; every lane
//    of the group then applies the same Newton step, so theta stays identical.
//  * Final pass: FP32 per-pixel Fisher products, summed per column in FP32
//    (<= 15 terms) and across columns and lanes in FP64; Cholesky (LU
//    fallback) inversion in FP64.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gmle {

struct KernelArgs {
    const float *data;      // (box, box, n) column-major
    const int32_t *xc;      // 1-based x (column) corners, may be null for Poisson
    const int32_t *yc;      // 1-based y (row) corners
    int64_t n;
    const float *var;       // (ny, nx) column-major variance map, e-^2
    const float *gain;      // (ny, nx) e-/ADU, used when adu != 0
    const float *offset;    // (ny, nx) ADU, used when adu != 0
    int32_t ny, nx;
    int32_t adu;            // 1: data are ADU, convert (ADU - offset) * gain
    int32_t iterations;
    int32_t tpr;            // threads per ROI: 1, 2, 4, 8, 16 or 32
    float sqrt2pi;          // sqrt(2f * Float32(pi)) as Julia evaluates it
    float psf[8];
    float lower[6], upper[6], max_step[6];
    float *params;          // [P, n]
    float *crlb;            // [P, n]
    float *llr;             // [n]
    uint8_t *flags;         // [n] or null
    unsigned long long *bad_corners;  // device counter of rejected ROIs
};

template <int MODEL> struct ModelInfo;
template <> struct ModelInfo<0> { static constexpr int P = 4; static constexpr bool SIG = false; };
template <> struct ModelInfo<1> { static constexpr int P = 5; static constexpr bool SIG = true; };
template <> struct ModelInfo<2> { static constexpr int P = 6; static constexpr bool SIG = true; };
template <> struct ModelInfo<3> { static constexpr int P = 5; static constexpr bool SIG = true; };

// Number of per-axis tables: psf, D1 (d/dpos), D2 (d2/dpos2) [, S1 (d/dsigma), S2].
template <int MODEL> __host__ __device__ constexpr int ntables() { return ModelInfo<MODEL>::SIG ? 5 : 3; }

constexpr uint8_t FLAG_CONVERGED = 1, FLAG_CHOLESKY = 2, FLAG_LU = 4, FLAG_SINGULAR = 8;

// ---- Julia scalar semantics -------------------------------------------------

// Base.clamp: ifelse(x > hi, hi, ifelse(x < lo, lo, x))  (NaN passes through)
__device__ __forceinline__ float jl_clamp(float x, float lo, float hi)
{
    return x > hi ? hi : (x < lo ? lo : x);
}
__device__ __forceinline__ float jl_maxf(float x, float y)
{
    if (isnan(x) || isnan(y)) return x + y;
    return signbit(x - y) ? y : x;
}
__device__ __forceinline__ double jl_maxd(double x, double y)
{
    if (isnan(x) || isnan(y)) return x + y;
    return signbit(x - y) ? y : x;
}
// Julia's Float32 x^4 and x^5 round a Float64 power_by_squaring once; the FP32
// products below are within 2 ulp of that and keep FP64 (1/64 of the FP32
// rate on GB300) out of the Newton loop.
__device__ __forceinline__ float jl_pow4f(float x)
{
    const float x2 = __fmul_rn(x, x);
    return __fmul_rn(x2, x2);
}
__device__ __forceinline__ float jl_pow5f(float x)
{
    return __fmul_rn(x, jl_pow4f(x));
}

// ---- per-axis coefficients (hoisted out of the pixel loops) ----------------

struct Axis {
    float c;     // centre (x or y, ROI pixels)
    float s;     // sigma (pixels)
    float sq;    // sqrt(0.5 / s^2): integral_gaussian_1d, baselibrary.jl:8-14
    float cst;   // (-N / sqrt(2pi)) / s: derivative_integral_gaussian_1d, baselibrary.jl:21-33
    float cst2;  // cst / s^2
    float s1c;   // ((-N / sqrt(2pi)) / s) / s: baselibrary.jl:40-52 (dudt)
    float s2c;   // (N / sqrt(2pi)) / s^5            (d2udt2 second term)
    float m2s;   // -2 / s                             (d2udt2 first factor)
};

__device__ __forceinline__ Axis make_axis(float c, float s, float N, float sqrt2pi, bool sig)
{
    Axis a;
    a.c = c;
    a.s = s;
    float s2 = __fmul_rn(s, s);
    a.sq = sqrtf(__fdiv_rn(0.5f, s2));
    float nk = __fdiv_rn(-N, sqrt2pi);
    a.cst = __fdiv_rn(nk, s);
    a.cst2 = __fdiv_rn(a.cst, s2);
    if (sig) {
        a.s1c = __fdiv_rn(a.cst, s);
        a.s2c = __fdiv_rn(__fdiv_rn(N, sqrt2pi), jl_pow5f(s));
        a.m2s = __fdiv_rn(-2.0f, s);
    } else {
        a.s1c = a.s2c = a.m2s = 0.f;
    }
    return a;
}

// Per-axis table entry at pixel index t (1-based).  psf: integral_gaussian_1d;
// d1, d2: derivative_integral_gaussian_1d without the PSF-of-the-other-axis
// factor; s1, s2: derivative_integral_gaussian_1d_sigma likewise.  The
// expressions keep the reference's association: (t - c) + 1/2 inside erf and
// the sigma products, (t + 1/2) - c inside exp.
template <bool SIG, bool SECOND>
__device__ __forceinline__ void axis_entry(int t, const Axis &a, float &psf, float &d1, float &d2,
                                           float &s1, float &s2)
{
    const float tf = (float)t;
    const float tc = tf - a.c;
    const float ua = __fadd_rn(tc, 0.5f), ub = __fadd_rn(tc, -0.5f);
    psf = 0.5f * (erff(__fmul_rn(ua, a.sq)) - erff(__fmul_rn(ub, a.sq)));
    const float ea = __fadd_rn(tf, 0.5f) - a.c, eb = __fadd_rn(tf, -0.5f) - a.c;
    const float ta = __fdiv_rn(ea, a.s), tb = __fdiv_rn(eb, a.s);
    const float fa = expf(-0.5f * __fmul_rn(ta, ta));
    const float fb = expf(-0.5f * __fmul_rn(tb, tb));
    d1 = a.cst * (fa - fb);
    if (SECOND) d2 = a.cst2 * (ea * fa - eb * fb);
    if (SIG) {
        s1 = a.s1c * (fa * ua - fb * ub);
        if (SECOND) s2 = a.s2c * (fa * (ua * ua * ua) - fb * (ub * ub * ub));
    }
}

// Astigmatic width model, src/psf_derivatives.jl:118-163 (per iteration, scalar).
struct AstigWidths {
    float sx, sy, dsx, dsy, d2sx, d2sy;
};

__device__ __forceinline__ void astig_widths(float z, const float *psf, AstigWidths &w)
{
    const float sx0 = psf[0], sy0 = psf[1], Ax = psf[2], Ay = psf[3], Bx = psf[4], By = psf[5];
    const float gam = psf[6], d = psf[7];
    const float zdx = __fdiv_rn(__fadd_rn(z, -gam), d);
    const float zdy = __fdiv_rn(__fadd_rn(z, gam), d);
    const float zdx2 = __fmul_rn(zdx, zdx), zdy2 = __fmul_rn(zdy, zdy);
    const float zdx3 = __fmul_rn(zdx2, zdx), zdy3 = __fmul_rn(zdy2, zdy);
    const float ax = __fadd_rn(__fadd_rn(__fadd_rn(1.0f, zdx2), __fmul_rn(Ax, zdx3)),
                               __fmul_rn(Bx, jl_pow4f(zdx)));
    const float ay = __fadd_rn(__fadd_rn(__fadd_rn(1.0f, zdy2), __fmul_rn(Ay, zdy3)),
                               __fmul_rn(By, jl_pow4f(zdy)));
    const float rax = sqrtf(ax), ray = sqrtf(ay);
    w.sx = __fmul_rn(sx0, rax);
    w.sy = __fmul_rn(sy0, ray);
    const float dax = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(2.0f, zdx), __fmul_rn(__fmul_rn(3.0f, Ax), zdx2)),
                                          __fmul_rn(__fmul_rn(4.0f, Bx), zdx3)), d);
    const float day = __fdiv_rn(__fadd_rn(__fadd_rn(__fmul_rn(2.0f, zdy), __fmul_rn(__fmul_rn(3.0f, Ay), zdy2)),
                                          __fmul_rn(__fmul_rn(4.0f, By), zdy3)), d);
    const float hx = __fdiv_rn(sx0, __fmul_rn(2.0f, rax));
    const float hy = __fdiv_rn(sy0, __fmul_rn(2.0f, ray));
    w.dsx = __fmul_rn(hx, dax);
    w.dsy = __fmul_rn(hy, day);
    const float dd = __fmul_rn(d, d);
    const float d2ax = __fdiv_rn(__fadd_rn(__fadd_rn(2.0f, __fmul_rn(__fmul_rn(6.0f, Ax), zdx)),
                                           __fmul_rn(__fmul_rn(12.0f, Bx), zdx2)), dd);
    const float d2ay = __fdiv_rn(__fadd_rn(__fadd_rn(2.0f, __fmul_rn(__fmul_rn(6.0f, Ay), zdy)),
                                           __fmul_rn(__fmul_rn(12.0f, By), zdy2)), dd);
    // alpha^1.5f0 (Julia rounds a Float64 pow once); alpha*sqrt(alpha) in FP32 is
    // within 1.5 ulp and avoids an FP64 pow per iteration.
    const float p15x = __fmul_rn(ax, rax);
    const float p15y = __fmul_rn(ay, ray);
    w.d2sx = __fadd_rn(__fmul_rn(-__fdiv_rn(sx0, __fmul_rn(4.0f, p15x)), __fmul_rn(dax, dax)),
                       __fmul_rn(hx, d2ax));
    w.d2sy = __fadd_rn(__fmul_rn(-__fdiv_rn(sy0, __fmul_rn(4.0f, p15y)), __fmul_rn(day, day)),
                       __fmul_rn(hy, d2ay));
}

// ---- group reductions --------------------------------------------------------

__device__ __forceinline__ float group_sum(float v, int tpr)
{
    for (int off = tpr >> 1; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}
__device__ __forceinline__ double group_sum(double v, int tpr)
{
    for (int off = tpr >> 1; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    return v;
}

// ---- initialisation, src/unified_kernel.jl:158-255 (one lane, reference order,
// no FMA contraction so that the start point matches the FP32 reference) ----

template <int MODEL, int BOX>
__device__ void initialize(const float *roi, const float *psf, float *th)
{
    float edge_sum = 0.f;
    int edge_count = 0;
    for (int j = 1; j <= BOX; j++)
        for (int i = 1; i <= BOX; i++)
            if (i == 1 || i == BOX || j == 1 || j == BOX) {
                edge_sum = __fadd_rn(edge_sum, roi[(i - 1) + BOX * (j - 1)]);
                edge_count++;
            }
    const float bg = __fdiv_rn(edge_sum, (float)edge_count);
    float total = 0.f, xw = 0.f, yw = 0.f;
    for (int j = 1; j <= BOX; j++)
        for (int i = 1; i <= BOX; i++) {
            const float sig = jl_maxf(0.f, __fadd_rn(roi[(i - 1) + BOX * (j - 1)], -bg));
            total = __fadd_rn(total, sig);
            xw = __fadd_rn(xw, __fmul_rn(sig, (float)j));
            yw = __fadd_rn(yw, __fmul_rn(sig, (float)i));
        }
    const float center = (float)((BOX + 1) / 2.0);
    float x = total > 10.f ? __fdiv_rn(xw, total) : center;
    float y = total > 10.f ? __fdiv_rn(yw, total) : center;
    x = jl_clamp(x, 1.5f, (float)(BOX - 0.5));
    y = jl_clamp(y, 1.5f, (float)(BOX - 0.5));
    const float photons = jl_maxf(total, 100.f);
    if (MODEL == 0) { th[0] = x; th[1] = y; th[2] = photons; th[3] = bg; }
    if (MODEL == 1) { th[0] = x; th[1] = y; th[2] = photons; th[3] = bg; th[4] = 1.3f; }
    if (MODEL == 2) { th[0] = x; th[1] = y; th[2] = photons; th[3] = bg; th[4] = 1.3f; th[5] = 1.3f; }
    if (MODEL == 3) {
        float tot2 = 0.f, mxx = 0.f, myy = 0.f;
        for (int j = 1; j <= BOX; j++)
            for (int i = 1; i <= BOX; i++) {
                const float sig = jl_maxf(0.f, __fadd_rn(roi[(i - 1) + BOX * (j - 1)], -bg));
                tot2 = __fadd_rn(tot2, sig);
                const float dx = __fadd_rn((float)j, -x), dy = __fadd_rn((float)i, -y);
                mxx = __fadd_rn(mxx, __fmul_rn(__fmul_rn(sig, dx), dx));
                myy = __fadd_rn(myy, __fmul_rn(__fmul_rn(sig, dy), dy));
            }
        float z = 0.f;
        if (tot2 > 10.f) {
            const float sxe = sqrtf(jl_maxf(0.5f, __fdiv_rn(mxx, tot2)));
            const float sye = sqrtf(jl_maxf(0.5f, __fdiv_rn(myy, tot2)));
            const float rx = __fdiv_rn(sxe, psf[0]), ry = __fdiv_rn(sye, psf[1]);
            const float da = __fadd_rn(__fmul_rn(rx, rx), -__fmul_rn(ry, ry));
            z = __fdiv_rn(__fmul_rn(-da, __fmul_rn(psf[7], psf[7])), __fmul_rn(4.0f, psf[6]));
            z = jl_clamp(z, -600.f, 600.f);
        }
        th[0] = x; th[1] = y; th[2] = z; th[3] = photons; th[4] = bg;
    }
}

// ---- FP64 CRLB from the Fisher matrix, src/unified_kernel.jl:399-431 --------

template <int P>
__device__ uint8_t crlb_from_fisher(double (&F)[P][P], float *crlb)
{
    double m = fabs(F[0][0]);
#pragma unroll
    for (int k = 0; k < P; k++)
#pragma unroll
        for (int l = 0; l < P; l++) m = jl_maxd(m, fabs(F[k][l]));
    const double reg = (double)1e-10f * m;
#pragma unroll
    for (int k = 0; k < P; k++) F[k][k] += reg;

    double L[P][P];
    bool ok = true;
    // static_cholesky_decomposition!, src/unified_kernel.jl:7-29
#pragma unroll
    for (int j = 0; j < P; j++) {
#pragma unroll
        for (int i = j; i < P; i++) {
            double s = F[i][j];
#pragma unroll
            for (int k = 0; k < j; k++) s -= L[i][k] * L[j][k];
            if (i == j) {
                if (!(s > 0.0) && !isnan(s)) ok = false;
                L[i][i] = sqrt(s);
            } else {
                L[i][j] = s / L[j][j];
            }
        }
    }
    double diag[P];
    uint8_t flags;
    if (ok) {
        // static_cholesky_inverse!, src/unified_kernel.jl:32-60 (diagonal only)
        double Li[P][P];
#pragma unroll
        for (int j = 0; j < P; j++) {
            Li[j][j] = 1.0 / L[j][j];
#pragma unroll
            for (int i = j + 1; i < P; i++) {
                double s = 0.0;
#pragma unroll
                for (int k = j; k < i; k++) s += L[i][k] * Li[k][j];
                Li[i][j] = -s / L[i][i];
            }
        }
#pragma unroll
        for (int i = 0; i < P; i++) {
            double s = 0.0;
#pragma unroll
            for (int k = i; k < P; k++) s += Li[k][i] * Li[k][i];
            diag[i] = s;
        }
        flags = FLAG_CHOLESKY;
    } else {
        // static_lu_decomposition! + static_matrix_inverse!, src/unified_kernel.jl:64-137
        double A[P][P];
        double am = 0.0;
#pragma unroll
        for (int k = 0; k < P; k++)
#pragma unroll
            for (int l = 0; l < P; l++) {
                A[k][l] = F[k][l];
                am = (k == 0 && l == 0) ? fabs(A[0][0]) : jl_maxd(am, fabs(A[k][l]));
            }
        const double tol = (double)1e-10f * am;
        bool lu_ok = true;
#pragma unroll
        for (int k = 0; k < P; k++) {
            if (fabs(A[k][k]) < tol) lu_ok = false;
#pragma unroll
            for (int i = k + 1; i < P; i++) {
                A[i][k] /= A[k][k];
#pragma unroll
                for (int j = k + 1; j < P; j++) A[i][j] -= A[i][k] * A[k][j];
            }
        }
        if (lu_ok) {
#pragma unroll
            for (int col = 0; col < P; col++) {
                double x[P];
#pragma unroll
                for (int i = 0; i < P; i++) {
                    x[i] = (i == col) ? 1.0 : 0.0;
#pragma unroll
                    for (int j = 0; j < i; j++) x[i] -= A[i][j] * x[j];
                }
#pragma unroll
                for (int i = P - 1; i >= 0; i--) {
#pragma unroll
                    for (int j = i + 1; j < P; j++) x[i] -= A[i][j] * x[j];
                    x[i] /= A[i][i];
                }
                diag[col] = x[col];
            }
            flags = FLAG_LU;
        } else {
#pragma unroll
            for (int k = 0; k < P; k++) diag[k] = __longlong_as_double(0x7ff0000000000000LL);
            flags = FLAG_SINGULAR;
        }
    }
#pragma unroll
    for (int k = 0; k < P; k++) {
        const double v = (flags == FLAG_SINGULAR) ? diag[k] : sqrt(jl_maxd(0.0, diag[k]));
        crlb[k] = (float)v;
    }
    if (isfinite(crlb[0])) flags |= FLAG_CONVERGED;
    return flags;
}

// ---- the kernel ---------------------------------------------------------------

// Shared memory per ROI slot: [BOX^2 data][BOX^2 variance if SCMOS][ok flag]
// [NT * BOX y-tables, only when tpr > 1], laid out as arrays over the R slots.
inline size_t smem_bytes(int model, int box, bool scmos, int tpr, int rois)
{
    const int nt = model == 0 ? 3 : 5;
    return (size_t)rois * (sizeof(float) * ((size_t)box * box * (scmos ? 2 : 1) +
                                            (tpr > 1 ? (size_t)nt * box : 0)) +
                           sizeof(int));
}

template <int MODEL, int BOX, bool SCMOS>
__global__ void __launch_bounds__(256) fit_kernel(const KernelArgs a)
{
    constexpr int P = ModelInfo<MODEL>::P;
    constexpr bool SIG = ModelInfo<MODEL>::SIG;
    constexpr int B2 = BOX * BOX;
    constexpr int NT = ntables<MODEL>();

    extern __shared__ __align__(16) float smem[];
    const int tpr = a.tpr;
    const int R = blockDim.x / tpr;
    float *sdata = smem;
    float *svar = sdata + R * B2;
    int *sok = reinterpret_cast<int *>(svar + (SCMOS ? R * B2 : 0));
    float *sytab = reinterpret_cast<float *>(sok + R);

    const int64_t roi0 = (int64_t)blockIdx.x * R;
    const int64_t left = a.n - roi0;
    const int nroi = left < R ? (int)left : R;

    // ---- stage the block's ROIs (contiguous in global memory) ----
    {
        const float *src = a.data + roi0 * B2;
        const int cnt = nroi * B2;
        if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
            const int c4 = cnt >> 2;
            const float4 *s4 = reinterpret_cast<const float4 *>(src);
            float4 *d4 = reinterpret_cast<float4 *>(sdata);
            for (int e = threadIdx.x; e < c4; e += blockDim.x) d4[e] = __ldg(s4 + e);
            for (int e = (c4 << 2) + threadIdx.x; e < cnt; e += blockDim.x) sdata[e] = __ldg(src + e);
        } else {
            for (int e = threadIdx.x; e < cnt; e += blockDim.x) sdata[e] = __ldg(src + e);
        }
        for (int e = cnt + threadIdx.x; e < R * B2; e += blockDim.x) sdata[e] = 0.f;
        for (int g = threadIdx.x; g < R; g += blockDim.x) {
            int ok = g < nroi;
            if (SCMOS && ok) {
                const int32_t x0 = a.xc[roi0 + g], y0 = a.yc[roi0 + g];
                ok = x0 >= 1 && y0 >= 1 && x0 + BOX - 1 <= a.nx && y0 + BOX - 1 <= a.ny;
                if (!ok) atomicAdd(a.bad_corners, 1ull);
            }
            sok[g] = ok;
        }
    }
    if (SCMOS) {
        __syncthreads();
        // gather the variance tile (and gain/offset for ADU data) of every ROI;
        // consecutive e walk down a column, i.e. contiguous map addresses.
        for (int e = threadIdx.x; e < R * B2; e += blockDim.x) {
            const int g = e / B2, p = e - g * B2;
            float v = 0.f;
            if (sok[g]) {
                const int j = p / BOX, i = p - j * BOX;
                const int64_t m = (int64_t)(a.yc[roi0 + g] - 1 + i) +
                                  (int64_t)a.ny * (int64_t)(a.xc[roi0 + g] - 1 + j);
                v = __ldg(a.var + m);
                if (a.adu) sdata[e] = __fmul_rn(__fadd_rn(sdata[e], -__ldg(a.offset + m)), __ldg(a.gain + m));
            }
            svar[e] = v;
        }
    }
    __syncthreads();

    const int g = threadIdx.x / tpr;  // ROI slot in the block
    const int r = threadIdx.x - g * tpr;
    const int lane = threadIdx.x & 31;
    const int leader = lane & ~(tpr - 1);
    // Warps without any ROI leave now (no block-wide barrier follows).
    if (__all_sync(0xffffffffu, g >= nroi)) return;
    const bool valid = g < nroi && sok[g];
    const float *roi = sdata + g * B2;
    const float *vroi = svar + g * B2;
    float *ytab = sytab + g * NT * BOX;

    float th[P];
#pragma unroll
    for (int k = 0; k < P; k++) th[k] = 0.f;
    if (r == 0) initialize<MODEL, BOX>(roi, a.psf, th);
#pragma unroll
    for (int k = 0; k < P; k++) th[k] = __shfl_sync(0xffffffffu, th[k], leader);

    float lo[P], hi[P], ms[P];
#pragma unroll
    for (int k = 0; k < P; k++) { lo[k] = a.lower[k]; hi[k] = a.upper[k]; ms[k] = a.max_step[k]; }

    // parameter slots
    constexpr int IX = 0, IY = 1;
    constexpr int IN = (MODEL == 3) ? 3 : 2;
    constexpr int IB = (MODEL == 3) ? 4 : 3;

    float yp[BOX], yd1[BOX], yd2[BOX], ys1[SIG ? BOX : 1], ys2[SIG ? BOX : 1];

    for (int it = 0; it <= a.iterations; ++it) {
        const bool final_pass = (it == a.iterations);
        // widths along x and y for this theta
        float sxw, syw;
        AstigWidths aw;
        if (MODEL == 0) { sxw = syw = a.psf[0]; }
        else if (MODEL == 1) { sxw = syw = th[4]; }
        else if (MODEL == 2) { sxw = th[4]; syw = th[5]; }
        else { astig_widths(th[2], a.psf, aw); sxw = aw.sx; syw = aw.sy; }
        const float N = th[IN], bg = th[IB];
        const Axis ax = make_axis(th[IX], sxw, N, a.sqrt2pi, SIG);
        const Axis ay = make_axis(th[IY], syw, N, a.sqrt2pi, SIG);

        // ---- y-axis tables (rows), held in registers ----
        if (tpr == 1) {
#pragma unroll
            for (int t = 0; t < BOX; t++) {
                float s1 = 0.f, s2 = 0.f;
                axis_entry<SIG, true>(t + 1, ay, yp[t], yd1[t], yd2[t], s1, s2);
                if (SIG) { ys1[t] = s1; ys2[t] = s2; }
            }
        } else {
            for (int t = r; t < BOX; t += tpr) {
                float p, d1, d2, s1 = 0.f, s2 = 0.f;
                axis_entry<SIG, true>(t + 1, ay, p, d1, d2, s1, s2);
                ytab[t] = p; ytab[BOX + t] = d1; ytab[2 * BOX + t] = d2;
                if (SIG) { ytab[3 * BOX + t] = s1; ytab[4 * BOX + t] = s2; }
            }
            __syncwarp();
#pragma unroll
            for (int t = 0; t < BOX; t++) {
                yp[t] = ytab[t]; yd1[t] = ytab[BOX + t]; yd2[t] = ytab[2 * BOX + t];
                if (SIG) { ys1[t] = ytab[3 * BOX + t]; ys2[t] = ytab[4 * BOX + t]; }
            }
            __syncwarp();
        }

        if (!final_pass) {
            // ---- gradient and diagonal Hessian (src/unified_kernel.jl:314-334) ----
            float gs[P], hs[P];
#pragma unroll
            for (int k = 0; k < P; k++) { gs[k] = 0.f; hs[k] = 0.f; }
            for (int j = r + 1; j <= BOX; j += tpr) {
                float xp, xd1, xd2, xs1 = 0.f, xs2 = 0.f;
                axis_entry<SIG, true>(j, ax, xp, xd1, xd2, xs1, xs2);
                const float npx = N * xp;
                const float *col = roi + (j - 1) * BOX;
                const float *vcol = vroi + (j - 1) * BOX;
#pragma unroll
                for (int t = 0; t < BOX; t++) {
                    const float py = yp[t];
                    const float mu = fmaf(npx, py, bg);
                    const float d = col[t];
                    float cf, df;
                    if (!SCMOS) {
                        if (mu > 0.01f) {
                            cf = fminf(__fdiv_rn(d, mu) - 1.0f, 1e4f);
                            df = fminf(__fdiv_rn(d, mu * mu), 1e4f);
                        } else {
                            cf = 0.f; df = 0.f;
                        }
                    } else {
                        const float tv = mu + vcol[t];
                        cf = __fdiv_rn(d - mu, tv);
                        df = __fdiv_rn(1.0f, tv);
                    }
                    // dudt and diagonal d2udt2 of src/psf_derivatives.jl
                    const float dux = xd1 * py, d2x = xd2 * py;
                    const float duy = yd1[t] * xp, d2y = yd2[t] * xp;
                    const float dun = xp * py;
                    gs[IX] = fmaf(dux, cf, gs[IX]);
                    hs[IX] += d2x * cf - dux * dux * df;
                    gs[IY] = fmaf(duy, cf, gs[IY]);
                    hs[IY] += d2y * cf - duy * duy * df;
                    gs[IN] = fmaf(dun, cf, gs[IN]);
                    hs[IN] -= dun * dun * df;
                    gs[IB] += cf;
                    hs[IB] -= df;
                    if (SIG) {
                        const float dsx = xs1 * py;
                        const float ddsx = ax.m2s * dsx - xs2 * py;
                        const float dsy = ys1[t] * xp;
                        const float ddsy = ay.m2s * dsy - ys2[t] * xp;
                        if (MODEL == 1) {
                            const float du = dsx + dsy, d2 = ddsx + ddsy;
                            gs[4] = fmaf(du, cf, gs[4]);
                            hs[4] += d2 * cf - du * du * df;
                        } else if (MODEL == 2) {
                            gs[4] = fmaf(dsx, cf, gs[4]);
                            hs[4] += ddsx * cf - dsx * dsx * df;
                            gs[5] = fmaf(dsy, cf, gs[5]);
                            hs[5] += ddsy * cf - dsy * dsy * df;
                        } else {
                            const float du = dsx * aw.dsx + dsy * aw.dsy;
                            const float d2 = ddsx * (aw.dsx * aw.dsx) + dsx * aw.d2sx +
                                             ddsy * (aw.dsy * aw.dsy) + dsy * aw.d2sy;
                            gs[2] = fmaf(du, cf, gs[2]);
                            hs[2] += d2 * cf - du * du * df;
                        }
                    }
                }
            }
            // ---- group reduction + scalar Newton step (src/unified_kernel.jl:337-350,
            //      apply_constraints!, src/constraints.jl:49-53) ----
#pragma unroll
            for (int k = 0; k < P; k++) {
                const float G = group_sum(gs[k], tpr);
                const float H = group_sum(hs[k], tpr);
                const float delta = fabsf(H) > 1e-10f ? __fdiv_rn(G, H) : 0.f;
                const float step = jl_clamp(delta, -ms[k], ms[k]);
                th[k] = jl_clamp(__fadd_rn(th[k], -step), lo[k], hi[k]);
            }
        } else {
            // ---- final pass: LLR + Fisher (src/unified_kernel.jl:354-397) ----
            float llr = 0.f;
            double F[P][P];
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = 0; l < P; l++) F[k][l] = 0.0;
            for (int j = r + 1; j <= BOX; j += tpr) {
                float xp, xd1, xd2, xs1 = 0.f, xs2 = 0.f;
                axis_entry<SIG, false>(j, ax, xp, xd1, xd2, xs1, xs2);
                const float npx = N * xp;
                const float *col = roi + (j - 1) * BOX;
                const float *vcol = vroi + (j - 1) * BOX;
                float S[P][P];
#pragma unroll
                for (int k = 0; k < P; k++)
#pragma unroll
                    for (int l = k; l < P; l++) S[k][l] = 0.f;
#pragma unroll
                for (int t = 0; t < BOX; t++) {
                    const float py = yp[t];
                    const float mu = fmaf(npx, py, bg);
                    const float d = col[t];
                    if (!SCMOS) {
                        if (mu > 0.f && d > 0.f)
                            llr += d * logf(mu) - mu - (d * logf(d) - d);
                        else if (mu > 0.f && d == 0.f)
                            llr -= mu;
                    } else {
                        const float tv = mu + vcol[t];
                        if (tv > 0.f) {
                            const float res = d - mu;
                            llr += -0.5f * __fdiv_rn(res * res, tv);
                        }
                    }
                    if (mu > 0.f) {
                        const float w = __fdiv_rn(1.0f, SCMOS ? mu + vcol[t] : mu);
                        float du[P];
                        du[IX] = xd1 * py;
                        du[IY] = yd1[t] * xp;
                        du[IN] = xp * py;
                        du[IB] = 1.0f;
                        if (MODEL == 1) du[4] = xs1 * py + ys1[t] * xp;
                        if (MODEL == 2) { du[4] = xs1 * py; du[5] = ys1[t] * xp; }
                        if (MODEL == 3) du[2] = (xs1 * py) * aw.dsx + (ys1[t] * xp) * aw.dsy;
#pragma unroll
                        for (int k = 0; k < P; k++) {
                            const float dkw = du[k] * w;
#pragma unroll
                            for (int l = k; l < P; l++) S[k][l] = fmaf(dkw, du[l], S[k][l]);
                        }
                    }
                }
#pragma unroll
                for (int k = 0; k < P; k++)
#pragma unroll
                    for (int l = k; l < P; l++) F[k][l] += (double)S[k][l];
            }
            llr = group_sum(llr, tpr);
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = k; l < P; l++) {
                    F[k][l] = group_sum(F[k][l], tpr);
                    F[l][k] = F[k][l];
                }
            if (r == 0 && valid) {
                const int64_t roi = roi0 + g;
                float cr[P];
                const uint8_t fl = crlb_from_fisher<P>(F, cr);
#pragma unroll
                for (int k = 0; k < P; k++) {
                    a.params[roi * P + k] = th[k];
                    a.crlb[roi * P + k] = cr[k];
                }
                a.llr[roi] = llr;
                if (a.flags) a.flags[roi] = fl;
            } else if (r == 0 && g < nroi) {
                // corner outside the calibration map: no fit
                const int64_t roi = roi0 + g;
                const float qnan = __int_as_float(0x7fc00000);
#pragma unroll
                for (int k = 0; k < P; k++) { a.params[roi * P + k] = qnan; a.crlb[roi * P + k] = qnan; }
                a.llr[roi] = qnan;
                if (a.flags) a.flags[roi] = 0;
            }
        }
    }
}

}  // namespace gmle
