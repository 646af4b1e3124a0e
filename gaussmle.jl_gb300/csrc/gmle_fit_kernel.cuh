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
//  * `tpr` lanes (1, 2, 4 or 8) fit one ROI; with several, each lane owns a
//    block of pixel columns and rows.  Per Newton iteration the model is
//    separable: per axis the erf/exp terms are evaluated once per pixel edge
//    (box + 1 per axis instead of 4 per pixel) into tables held in registers,
//    and per pixel only the likelihood terms are formed and summed into
//    per-column and per-row sums.
//  * With several lanes, the gradient and diagonal Hessian are summed with
//    warp shuffles; every lane of the group then applies the same Newton
//    step, so theta stays identical.
//  * Final pass: FP32 per-pixel Fisher products, summed per column in FP32
//    (<= 15 terms) and across columns and lanes as a compensated double-float
//    (FP64-class accuracy at FP32 cost); Cholesky (LU fallback) inversion in
//    FP64.
#pragma once

#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include <type_traits>

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

// Group table of a table launch.  A table launch fits every group of one
// (PSF model, box size, camera family) of a mixed batch: its groups' ROIs are
// cut into tiles of rois_per_block ROIs, numbered group after group.  With a
// `counter`, a persistent grid takes tiles from it (work stealing) until none
// is left; without one, the grid has one block per tile and block b fits tile
// b, so that each block frees its resources (tensor memory included) after
// one tile and concurrent launches interleave like plain launches.  With
// `tiles`, entry t is (group << 32) | (tile index within the group); without
// it, the tile's group is found by binary search of `tile0` (first tile of
// each group, increasing).
struct TileTable {
    const int64_t *header;        // [0] groups, [1] tiles; nullptr: plain launch
    const KernelArgs *groups;     // per group: its kernel arguments
    const int64_t *tiles;         // per tile: (group << 32) | local tile, or nullptr
    const int64_t *tile0;         // per group: first tile (used when tiles is nullptr)
    unsigned long long *counter;  // next tile, zero when the launch starts; nullptr:
                                  // one block per tile
};

template <int MODEL> struct ModelInfo;
template <> struct ModelInfo<0> { static constexpr int P = 4; static constexpr bool SIG = false; };
template <> struct ModelInfo<1> { static constexpr int P = 5; static constexpr bool SIG = true; };
template <> struct ModelInfo<2> { static constexpr int P = 6; static constexpr bool SIG = true; };
template <> struct ModelInfo<3> { static constexpr int P = 5; static constexpr bool SIG = true; };


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

// ---- fast elementary functions -----------------------------------------------
//
// The library's erff costs 28 issued instructions, expf 9 and __fdividef(1, x)
// 4 on GB300; the fit evaluates them per pixel edge and per pixel.  These
// replacements use single SFU instructions (PTX rcp.approx / ex2.approx,
// flush-to-zero: subnormal results are 0) and, for erf, the exponential that
// the fit already evaluates at the same pixel edge.

// 1/x, within 1 ulp
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// 2^x, within 2 ulp
__device__ __forceinline__ float ex2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
// ln(x) = log2(x) * ln 2 (PTX lg2.approx, subnormal inputs kept: about 2^-22
// absolute in log2, i.e. within a few ulp of ln for the photon counts and
// model values the Poisson LLR takes; the library's logf costs 26 issued
// instructions, and the final pass takes two per pixel)
__device__ __forceinline__ float log_approx(float x)
{
    float r;
    asm("lg2.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r * 0.69314718055994531f;
}
// exp(-t^2 / 2) = 2^(t^2 * (-log2(e) / 2)); the rounding of the exponent
// costs at most |t^2| 2^-23 relative, i.e. nothing where the value matters.
__device__ __forceinline__ float gauss_edge(float t)
{
    return ex2_approx(__fmul_rn(t, t) * -0.72134752044448170368f);
}
// erf(x), given e = exp(-x^2) (the caller's gauss_edge at the same edge).
// Hastings' form (Abramowitz & Stegun 7.1.26): erf(|x|) = 1 - e t P(t) with
// t = 1 / (1 + p |x|), here with P of degree 5 refitted by a least-squares
// (Lawson) minimax fit of exp(-x^2) erfcx(x) on [0, 6]: p = 0.39, 8.3e-9 largest
// error in exact arithmetic, below 4e-7 absolute evaluated in FP32 (most of it
// near x = 0, from 1 - e t P(t)); erf(-x) = -erf(x).  Checked against the
// library's erff by tests/test_math_gpu.py.
__device__ __forceinline__ float erf_from_gauss(float x, float e)
{
    const float t = rcp_approx(fmaf(0.39f, fabsf(x), 1.0f));
    float p = -0.22753699123859406f;
    p = fmaf(p, t, 0.8866637945175171f);
    p = fmaf(p, t, -0.6353994011878967f);
    p = fmaf(p, t, 0.6495586633682251f);
    p = fmaf(p, t, 0.09138870239257812f);
    p = fmaf(p, t, 0.2353251725435257f);
    return copysignf(fmaf(-e, t * p, 1.0f), x);
}

// ---- per-axis coefficients (hoisted out of the pixel loops) ----------------

struct Axis {
    float c;     // centre (x or y, ROI pixels)
    float s;     // sigma (pixels)
    float inv_s; // 1 / s
    float sq;    // sqrt(0.5 / s^2): integral_gaussian_1d, baselibrary.jl:8-14
    float cst;   // (-N / sqrt(2pi)) / s: derivative_integral_gaussian_1d, baselibrary.jl:21-33
    float cst2;  // cst / s^2
    float s1c;   // ((-N / sqrt(2pi)) / s) / s: baselibrary.jl:40-52 (dudt)
    float s2c;   // (N / sqrt(2pi)) / s^5            (d2udt2 second term)
    float m2s;   // -2 / s                             (d2udt2 first factor)
};

__device__ __forceinline__ Axis make_axis(float c, float s, float N, float sqrt2pi, bool sig)
{
    // One division per axis; the remaining factors are products of 1/s, each
    // within a few ulp of the reference's chained divisions.
    Axis a;
    a.c = c;
    a.s = s;
    const float is = __fdiv_rn(1.0f, s);
    a.inv_s = is;
    const float is2 = is * is;
    a.sq = 0.70710678118654752f * is;                 // sqrt(1/2 / s^2), s > 0
    const float nk = -N * __fdiv_rn(1.0f, sqrt2pi);   // -N / sqrt(2 pi)
    a.cst = nk * is;
    a.cst2 = a.cst * is2;
    if (sig) {
        a.s1c = a.cst * is;
        a.s2c = -nk * (is2 * is2 * is);
        a.m2s = -2.0f * is;
    } else {
        a.s1c = a.s2c = a.m2s = 0.f;
    }
    return a;
}

// Table entries of consecutive pixel indices along one axis.  Neighbouring
// pixels share an edge: the exp at the upper edge of pixel t is the exp at the
// lower edge of pixel t+1 (both arguments are the same float, (t + 1/2) - c),
// and the erf at the upper edge, ((t - c) + 1/2) * sq, is reused as the lower
// edge of t+1, ((t + 1 - c) - 1/2) * sq, whenever the two arguments are equal
// (always, unless t - c rounds; then the lower edge is evaluated).  A run of
// pixels costs about one erf and one exp per pixel instead of two of each.
struct EdgeWalk {
    float ua;    // erf-argument offset (t - c) + 1/2 of the previous pixel's upper edge
    float erfa;  // erf(ua * sq)
    float ea;    // exp-argument offset (t + 1/2) - c of the previous pixel's upper edge
    float fa;    // exp at the previous pixel's upper edge
};

// Start a walk at pixel t0: the values of its lower edge.
__device__ __forceinline__ EdgeWalk walk_start(int t0, const Axis &a)
{
    const float tf = (float)t0;
    const float ub = __fadd_rn(tf - a.c, -0.5f);
    const float eb = __fadd_rn(tf, -0.5f) - a.c;
    EdgeWalk w;
    w.ua = ub;
    w.ea = eb;
    w.fa = gauss_edge(eb * a.inv_s);
    w.erfa = erf_from_gauss(__fmul_rn(ub, a.sq), w.fa);
    return w;
}

// psf: integral_gaussian_1d (baselibrary.jl:8-14); d1, d2:
// derivative_integral_gaussian_1d (baselibrary.jl:21-33) and s1, s2:
// derivative_integral_gaussian_1d_sigma (baselibrary.jl:40-52), each without
// the factor PSF of the other axis.  The expressions keep the reference's
// association: (t - c) + 1/2 inside erf and the sigma products, (t + 1/2) - c
// inside exp.
//
// VOTE (one-thread-per-ROI kernel only, where a warp's 32 lanes walk in step):
// the rare re-evaluation of the lower edge's erf sits behind a warp vote, so
// that it costs issue slots only in the warps that need it.  Measured per
// kernel (plain launches, sCMOS ADU): astigmatic 15x15 1.874 -> 1.815 ms for
// 300 000 ROIs, XYNB 7x7 0.153 -> 0.151 ms for 100 000; slower for
// XYNBSXSY 13x13 (1.331 -> 1.382 ms), XYNB 11x11 (1.791 -> 1.804 ms) and the
// astigmatic 15x15 Poisson kernel.
template <bool SIG, bool SECOND, bool VOTE = false>
__device__ __forceinline__ void walk_entry(int t, const Axis &a, EdgeWalk &w, float &psf,
                                           float &d1, float &d2, float &s1, float &s2)
{
    const float tf = (float)t;
    const float tc = tf - a.c;
    const float ua = __fadd_rn(tc, 0.5f), ub = __fadd_rn(tc, -0.5f);
    // the lower edge's exp argument (t - 1/2) - c is the previous upper edge's
    // ((t - 1) + 1/2) - c: the same two operands, the same float
    const float ea = __fadd_rn(tf, 0.5f) - a.c, eb = w.ea;
    const float fb = w.fa;
    const float fa = gauss_edge(ea * a.inv_s);
    float erfb = w.erfa;
    if (VOTE) {
        if (__any_sync(0xffffffffu, ub != w.ua)) {
            const float r = erf_from_gauss(__fmul_rn(ub, a.sq), fb);
            erfb = ub != w.ua ? r : erfb;
        }
    } else if (ub != w.ua) {
        erfb = erf_from_gauss(__fmul_rn(ub, a.sq), fb);
    }
    const float erfa = erf_from_gauss(__fmul_rn(ua, a.sq), fa);
    // the true value is >= 0 (erf is increasing and ua > ub), so is the
    // reference's; a negative rounding residue of the tails is cut to 0
    psf = fmaxf(0.5f * (erfa - erfb), 0.0f);
    d1 = a.cst * (fa - fb);
    if (SECOND) d2 = a.cst2 * (ea * fa - eb * fb);
    if (SIG) {
        s1 = a.s1c * (fa * ua - fb * ub);
        if (SECOND) s2 = a.s2c * (fa * (ua * ua * ua) - fb * (ub * ub * ub));
    }
    w.ua = ua;
    w.erfa = erfa;
    w.ea = ea;
    w.fa = fa;
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

// ---- compensated (double-float) accumulation of the Fisher matrix ------------
//
// A value is an unevaluated sum hi + lo of two floats.  TwoSum (Moller 1965,
// Knuth TAOCP vol. 2, 4.2.2) gives the exact rounding error of a float
// addition in 6 additions, so the accumulated sum of FP32 terms is carried to
// about 2^-48 relative, like an FP64 accumulator, at FP32 cost: FP64 runs at
// 1/64 of the FP32 rate on GB300.  The sum becomes a double (hi + lo, exact)
// for the FP64 inversion.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fadd_rn(s, -a);
    e = __fadd_rn(__fadd_rn(a, -__fadd_rn(s, -bb)), __fadd_rn(b, -bb));
}

// hi + lo += x
__device__ __forceinline__ void dd_add(float &hi, float &lo, float x)
{
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo = __fadd_rn(lo, e);
}

// (hi, lo) summed over the tpr lanes of a group (all lanes get the same sum:
// TwoSum's error term is exact, so it does not depend on the operand order).
__device__ __forceinline__ void dd_group_sum(float &hi, float &lo, int tpr)
{
    for (int off = tpr >> 1; off > 0; off >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, hi, off);
        const float ol = __shfl_xor_sync(0xffffffffu, lo, off);
        float s, e;
        two_sum(hi, oh, s, e);
        e = __fadd_rn(e, __fadd_rn(lo, ol));
        two_sum(s, e, hi, lo);  // renormalise: |lo| <= ulp(hi) / 2
    }
}

__device__ __forceinline__ double dd_to_double(float hi, float lo)
{
    return __dadd_rn((double)hi, (double)lo);
}

// ---- initialisation, src/unified_kernel.jl:158-255 (one lane, reference order,
// no FMA contraction so that the start point matches the FP32 reference) ----

// roi(p) gives pixel p = (i - 1) + BOX (j - 1) of the ROI; BOX may be a
// compile-time constant (the specialised kernels) or the run-time box.
template <int MODEL, typename Roi>
__device__ __forceinline__ void initialize_box(const int BOX, Roi roi, const float *psf, float *th)
{
    float edge_sum = 0.f;
    int edge_count = 0;
    for (int j = 1; j <= BOX; j++)
        for (int i = 1; i <= BOX; i++)
            if (i == 1 || i == BOX || j == 1 || j == BOX) {
                edge_sum = __fadd_rn(edge_sum, roi((i - 1) + BOX * (j - 1)));
                edge_count++;
            }
    const float bg = __fdiv_rn(edge_sum, (float)edge_count);
    float total = 0.f, xw = 0.f, yw = 0.f;
    for (int j = 1; j <= BOX; j++)
        for (int i = 1; i <= BOX; i++) {
            const float sig = jl_maxf(0.f, __fadd_rn(roi((i - 1) + BOX * (j - 1)), -bg));
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
                const float sig = jl_maxf(0.f, __fadd_rn(roi((i - 1) + BOX * (j - 1)), -bg));
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

template <int MODEL, int BOX, int STRIDE>
__device__ void initialize(const float *roi_pix, const float *psf, float *th)
{
    // roi_pix holds the ROI's pixels STRIDE floats apart (2: (data, variance) pairs)
    initialize_box<MODEL>(BOX, [&](int p) { return roi_pix[STRIDE * p]; }, psf, th);
}

// ---- FP64 CRLB from the Fisher matrix, src/unified_kernel.jl:399-431 --------

template <int P>
__device__ uint8_t crlb_from_fisher(double (&F)[P][P], float *crlb)
{
    // max |F| (F is symmetric: its upper triangle).  The bit patterns of
    // non-negative doubles order like their values, and |NaN| orders above
    // +Inf, so an integer maximum of the magnitudes' bits is Julia's maximum,
    // NaN-propagating, computed on the integer pipe instead of FP64.
    long long mb = 0;
#pragma unroll
    for (int k = 0; k < P; k++)
#pragma unroll
        for (int l = k; l < P; l++)
            mb = max(mb, __double_as_longlong(F[k][l]) & 0x7fffffffffffffffLL);
    const double reg = (double)1e-10f * __longlong_as_double(mb);
#pragma unroll
    for (int k = 0; k < P; k++) F[k][k] += reg;

    // FP64 divisions and square roots are long instruction sequences on a pipe
    // that runs at 1/64 of the FP32 rate: each pivot takes one reciprocal
    // square root, rL[j] = 1 / L[j][j], and every division by a pivot becomes
    // a product with it (within an FP64 ulp or two of the divisions).
    double L[P][P], rL[P];
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
                rL[j] = rsqrt(s);
                L[j][j] = s * rL[j];
            } else {
                L[i][j] = s * rL[j];
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
            Li[j][j] = rL[j];
#pragma unroll
            for (int i = j + 1; i < P; i++) {
                double s = 0.0;
#pragma unroll
                for (int k = j; k < i; k++) s += L[i][k] * Li[k][j];
                Li[i][j] = -s * rL[i];
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
    // CRLB = sqrt(max(0, diag)): the output is Float32, so the root is taken
    // in FP32 of the rounded variance (within an FP32 ulp of the FP64 root)
#pragma unroll
    for (int k = 0; k < P; k++)
        crlb[k] = (flags == FLAG_SINGULAR) ? (float)diag[k]
                                           : sqrtf((float)jl_maxd(0.0, diag[k]));
    if (isfinite(crlb[0])) flags |= FLAG_CONVERGED;
    return flags;
}


// ---- shared pieces of the two kernels ----------------------------------------

// Shared memory, as arrays over the R ROI slots of a block: pixels (float, or
// float2 (data in e-, read-noise variance) for sCMOS), for sCMOS the map
// offset of each ROI's first pixel (int64), and one ok flag per slot.
//
// One thread per ROI (tpr == 1) keeps only the data plane in shared memory:
// with sCMOS data each thread's variance tile lives in its tensor-memory lane
// (TmemVar below), and its ROI's map offset and ok flag in its registers
// (stage_r1), so a ROI takes box^2 floats.
__host__ __device__ inline size_t smem_bytes(int model, int box, bool scmos, int tpr, int rois)
{
    (void)model;
    if (tpr == 1) return (size_t)rois * sizeof(float) * box * box;
    return (size_t)rois * (sizeof(float) * (size_t)box * box * (scmos ? 2 : 1) +
                           (scmos ? sizeof(long long) : 0) + sizeof(int));
}

// A table launch's block keeps, after the ROI slots, its current group's
// kernel arguments and the tile it works on.
struct TableSlot {
    KernelArgs a;
    long long tile;  // local tile index within the group; -1: no tile left
    int grp;         // group whose arguments `a` holds; -1: none yet
    int next;        // group of the tile just taken
};
__host__ __device__ inline size_t table_slot_offset(size_t smem) { return (smem + 15) & ~size_t(15); }
__host__ __device__ inline size_t table_smem_bytes(size_t smem)
{
    return table_slot_offset(smem) + sizeof(TableSlot);
}

__device__ __forceinline__ TableSlot *table_slot(float *smem, size_t smem_rois)
{
    return reinterpret_cast<TableSlot *>(reinterpret_cast<char *>(smem) +
                                         table_slot_offset(smem_rois));
}

__device__ __forceinline__ void table_slot_init(TableSlot *ts)
{
    if (threadIdx.x == 0) ts->grp = -1;
}

// The block's k-th tile of a table launch: thread 0 takes it from the counter
// (or, with one block per tile, tile blockIdx.x when k == 0 and none after)
// and finds its group; when the group changes, the block copies the group's
// arguments into the slot.  Returns false when no tile is left.  Ends with a
// barrier, so the slot is stable for the whole tile; the caller puts a
// barrier between the end of a tile and the next call.
__device__ __forceinline__ bool table_next(const TileTable &t, int R, TableSlot *ts, int k,
                                           int64_t &roi0, int &nroi)
{
    if (threadIdx.x == 0) {
        const long long tile = t.counter ? (long long)atomicAdd(t.counter, 1ull)
                               : k == 0  ? (long long)blockIdx.x
                                         : LLONG_MAX;
        int g = -1;
        long long local = -1;
        if (tile < t.header[1]) {
            if (t.tiles) {
                const int64_t e = t.tiles[tile];
                g = (int)(e >> 32);
                local = e & 0xffffffffLL;
            } else {
                // tiles are taken in increasing order: search from the block's group on
                int lo = ts->grp < 0 ? 0 : ts->grp, hi = (int)t.header[0] - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (t.tile0[mid] <= tile) lo = mid; else hi = mid - 1;
                }
                g = lo;
                local = tile - t.tile0[g];
            }
        }
        ts->tile = local;
        ts->next = g;
    }
    __syncthreads();
    const int g = ts->next;
    if (g < 0) return false;
    if (g != ts->grp) {
        const int *src = reinterpret_cast<const int *>(t.groups + g);
        int *dst = reinterpret_cast<int *>(&ts->a);
        for (int w = threadIdx.x; w < (int)(sizeof(KernelArgs) / sizeof(int)); w += blockDim.x)
            dst[w] = src[w];
        __syncthreads();  // the copy is complete and every thread has compared ts->grp
        if (threadIdx.x == 0) ts->grp = g;
    }
    roi0 = ts->tile * R;
    const int64_t left = ts->a.n - roi0;
    nroi = left < R ? (int)left : R;
    return true;
}

// Asynchronous global -> shared copies (cp.async, sm_80+ PTX); src_bytes = 0
// fills the destination with zeros without reading the source.
__device__ __forceinline__ void cp_async4(void *dst, const void *src, unsigned src_bytes)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(s), "l"(src),
                 "r"(src_bytes) : "memory");
}
// .ca, not .cg: from pinned host memory (ROI data the serving loop reads in
// place) 16-byte .cg copies ran at 93 GB/s on GB300, .ca copies, 4-byte
// copies and plain loads at the host link's 211 GB/s; from HBM they are alike.
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// ---- tensor memory (TMEM) as per-thread storage ------------------------------
//
// Blackwell's tensor memory (128 lanes x 512 32-bit columns per SM) is
// otherwise idle in this kernel.  The one-thread-per-ROI sCMOS kernel keeps
// each ROI's variance tile there: thread i of warp w owns TMEM lane
// 32 (w % 4) + i (a warp reaches only its lane quarter), pixel p of its ROI is
// column p of the CTA's allocation, and each fitted column is read back with
// one tcgen05.ld.  Allocation is by columns across all 128 lanes, so CTAs of
// four warps use it fully.  Warp 0 allocates at kernel start and frees it at
// kernel end, on every path; a CTA that finds TMEM full waits in
// tcgen05.alloc until a resident CTA frees its columns.
template <int BOX> struct TmemVar {
    static constexpr int B2 = BOX * BOX;
    static constexpr int LW = BOX <= 8 ? 8 : 16;  // columns of one per-column load
    static constexpr int CHUNKS = (B2 + 15) / 16;  // 16-column stores of a tile
    static constexpr int NEED = CHUNKS * 16 > BOX * (BOX - 1) + LW ? CHUNKS * 16
                                                                   : BOX * (BOX - 1) + LW;
    static constexpr int NCOLS = NEED <= 32 ? 32 : NEED <= 64 ? 64 : NEED <= 128 ? 128
                               : NEED <= 256 ? 256 : 512;
    static_assert(NEED <= 512, "variance tile larger than tensor memory");
};

__host__ __device__ constexpr int tmem_var_cols(int box)
{
    // TmemVar<box>::NCOLS for a run-time box
    const int b2 = box * box, lw = box <= 8 ? 8 : 16, chunks = (b2 + 15) / 16;
    const int need = chunks * 16 > box * (box - 1) + lw ? chunks * 16 : box * (box - 1) + lw;
    return need <= 32 ? 32 : need <= 64 ? 64 : need <= 128 ? 128 : need <= 256 ? 256 : 512;
}

template <int NCOLS>
__device__ __forceinline__ void tmem_alloc(uint32_t *s_dst)  // one full warp
{
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(s_dst);
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(dst), "n"(NCOLS) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
template <int NCOLS>
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr)  // one full warp
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(taddr), "n"(NCOLS) : "memory");
}
// Around a CTA barrier that orders tensor-memory accesses.
__device__ __forceinline__ void tmem_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// The tensor-memory load and store touch only registers and tensor memory, so
// they carry no "memory" clobber: global and shared accesses may move across
// them (the gathers of the next column ahead of this column's store, the
// pixel loads of a column ahead of its variance load).  Being volatile, they
// keep their order among themselves and with the fences and barriers.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const float (&v)[16])
{
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, "
                 "%8, %9, %10, %11, %12, %13, %14, %15, %16};"
                 :: "r"(taddr), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]),
                    "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]), "f"(v[10]), "f"(v[11]),
                    "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15]));
}
__device__ __forceinline__ void tmem_wait_st()
{
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
// Load LW (8 or 16) consecutive columns of this thread's lane; waits for them.
template <int LW>
__device__ __forceinline__ void tmem_ld(uint32_t taddr, float (&v)[LW])
{
    if constexpr (LW == 16) {
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, "
                     "%8, %9, %10, %11, %12, %13, %14, %15}, [%16];\n"
                     "tcgen05.wait::ld.sync.aligned;"
                     : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                       "=f"(v[6]), "=f"(v[7]), "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]),
                       "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
                     : "r"(taddr));
    } else {
        static_assert(LW == 8, "8 or 16 columns");
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, "
                     "[%8];\n"
                     "tcgen05.wait::ld.sync.aligned;"
                     : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                       "=f"(v[6]), "=f"(v[7])
                     : "r"(taddr));
    }
}

// The same load without its wait, and the wait: between them the registers
// are in flight and must not be read.  The wait takes them as in-out
// operands, so no read of them can move above it.
template <int LW>
__device__ __forceinline__ void tmem_ld_start(uint32_t taddr, float (&v)[LW])
{
    if constexpr (LW == 16) {
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, "
                     "%8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                     : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                       "=f"(v[6]), "=f"(v[7]), "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]),
                       "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
                     : "r"(taddr));
    } else {
        static_assert(LW == 8, "8 or 16 columns");
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                     : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]),
                       "=f"(v[6]), "=f"(v[7])
                     : "r"(taddr));
    }
}
template <int LW>
__device__ __forceinline__ void tmem_ld_wait(float (&v)[LW])
{
    if constexpr (LW == 16) {
        asm volatile("tcgen05.wait::ld.sync.aligned;"
                     : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]),
                       "+f"(v[6]), "+f"(v[7]), "+f"(v[8]), "+f"(v[9]), "+f"(v[10]), "+f"(v[11]),
                       "+f"(v[12]), "+f"(v[13]), "+f"(v[14]), "+f"(v[15]));
    } else {
        asm volatile("tcgen05.wait::ld.sync.aligned;"
                     : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]),
                       "+f"(v[6]), "+f"(v[7]));
    }
}

// ADU -> e- of the staged pixels (PS floats apart), (ADU - offset) * gain
// (src/camera_models.jl:110-113).  The gain and offset gathers (L2-resident
// maps) of kU pixels are issued before any is used, so that they overlap.
template <int BOX, int PS>
__device__ __forceinline__ void adu_to_electrons(const KernelArgs &a, float *spix, const int *sok,
                                                 const long long *sbase, int cnt)
{
    constexpr int B2 = BOX * BOX;
    constexpr int kU = 16;
    for (int e0 = threadIdx.x; e0 < cnt; e0 += kU * blockDim.x) {
        float off[kU], gn[kU];
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int e = e0 + u * blockDim.x;
            off[u] = 0.f;
            gn[u] = 1.f;
            const int g = e / B2;
            if (e < cnt && sok[g]) {
                const int p = e - g * B2, j = p / BOX, i = p - j * BOX;
                const long long m = sbase[g] + i + (long long)a.ny * j;
                off[u] = __ldg(a.offset + m);
                gn[u] = __ldg(a.gain + m);
            }
        }
#pragma unroll
        for (int u = 0; u < kU; u++) {
            const int e = e0 + u * blockDim.x;
            if (e < cnt && sok[e / B2])
                spix[PS * e] = __fmul_rn(__fadd_rn(spix[PS * e], -off[u]), gn[u]);
        }
    }
}

// Copy of the block's data plane, nroi ROIs of box^2 floats contiguous in
// global memory from `src`, to `spix` (16-byte cp.async where the source is
// aligned); slots [nroi, R) are zero-filled.  Waits for the thread's copies.
template <int BOX>
__device__ __forceinline__ void copy_data_plane(float *spix, const float *src, int R, int nroi)
{
    constexpr int B2 = BOX * BOX;
    const int cnt = nroi * B2;
    if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
        const int c4 = cnt >> 2;
        for (int e = threadIdx.x; e < c4; e += blockDim.x) cp_async16(spix + 4 * e, src + 4 * e);
        for (int e = (c4 << 2) + threadIdx.x; e < cnt; e += blockDim.x)
            cp_async4(spix + e, src + e, 4);
    } else {
        for (int e = threadIdx.x; e < cnt; e += blockDim.x) cp_async4(spix + e, src + e, 4);
    }
    for (int e = cnt + threadIdx.x; e < R * B2; e += blockDim.x) spix[e] = 0.f;
    cp_async_wait_all();
}

// One map column of a ROI, BOX consecutive floats of `map` from a0 + sh with
// a0 a multiple of 4 (so map + a0 is 16-byte aligned), by aligned float4
// loads: only the float4s that hold a pixel of the column (each lies inside
// the map, whose length is a multiple of 4), then the column's floats picked
// by two levels of selects on the bits of sh (0..3).  With `in` false
// nothing is loaded and the column is `fill`.
template <int BOX>
__device__ __forceinline__ void map_column4(const float *__restrict__ map, long long a0, int sh,
                                            bool in, float fill, float (&col)[BOX])
{
    constexpr int NQ = (BOX + 6) / 4;  // float4s for sh = 3: 4 NQ >= BOX + 3
    float f[4 * NQ];
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        float4 w = make_float4(fill, fill, fill, fill);
        if (in && (4 * q < BOX || 4 * q < sh + BOX))
            w = __ldg(reinterpret_cast<const float4 *>(map + a0) + q);
        f[4 * q] = w.x;
        f[4 * q + 1] = w.y;
        f[4 * q + 2] = w.z;
        f[4 * q + 3] = w.w;
    }
    const bool s0 = sh & 1, s1 = sh & 2;
    float t[BOX + 2];
#pragma unroll
    for (int i = 0; i < BOX + 2; i++) t[i] = s0 ? f[i + 1] : f[i];
#pragma unroll
    for (int i = 0; i < BOX; i++) col[i] = s1 ? t[i + 2] : t[i];
}

// Staging of the one-thread-per-ROI kernel.  Slot g = threadIdx.x of the
// block holds ROI roi0 + g.  Each lane first checks its own ROI's corners;
// the map offset and the ok flag stay in its registers, so a ROI takes only
// its pixels in shared memory.  sCMOS then needs, per ROI, its variance tile
// in the owning lane's tensor memory (pixel p at column p; zeros for an
// empty or rejected slot) and, for ADU data, its pixels converted in place,
// (ADU - offset) * gain (src/camera_models.jl:110-113; rejected ROIs stay as
// they are).  Two ways are compiled, by box size (each the faster one
// measured on GB300):
//
// * up to 11x11, per lane: the block copies its pixels, and after a barrier
//   each lane gathers its own ROI's variance, gain and offset.  When the maps
//   are 16-byte aligned with ny a multiple of 4, every column of a ROI starts
//   at the same offset (y0 - 1) mod 4 within a float4, so each column is
//   read by a few aligned float4 loads instead of box scalar loads
//   (map_column4); otherwise by scalar loads, 16 pixels' worth issued before
//   any is used.
// * 13x13 and 15x15, per warp, with no block barrier: warp w stages its own
//   32 slots.  The variance tiles are copied from the map into the ROIs'
//   shared-memory slots by 4-byte cp.async, two ROI columns per instruction
//   (lanes 0-15 column j, 16-31 column j + 1), so consecutive lanes read
//   consecutive map rows; each lane then moves its slot into its
//   tensor-memory lane; then the warp's pixels are copied over the slots and
//   converted with the same coalesced gathers of gain and offset.  The ROI
//   whose map offset a step needs comes from its lane by a warp shuffle.
//
// Every thread of the block calls it (the tensor-memory stores are
// warp-wide).  Returns whether slot threadIdx.x holds a ROI with valid
// corners.
template <int BOX, bool SCMOS>
__device__ __forceinline__ bool stage_r1(const KernelArgs &a, float *spix, int64_t roi0,
                                         int nroi, uint32_t taddr)
{
    constexpr int B2 = BOX * BOX;
    if constexpr (!SCMOS || BOX <= 11) {
        copy_data_plane<BOX>(spix, a.data + roi0 * B2, blockDim.x, nroi);
        __syncthreads();  // other threads' copies of this thread's ROI
        const int g = threadIdx.x;
        bool ok = g < nroi;
        if (!SCMOS) return ok;
        long long base = 0;
        if (ok) {
            const int32_t x0 = a.xc[roi0 + g], y0 = a.yc[roi0 + g];
            ok = x0 >= 1 && y0 >= 1 && x0 + BOX - 1 <= a.nx && y0 + BOX - 1 <= a.ny;
            if (!ok) atomicAdd(a.bad_corners, 1ull);
            base = ok ? (long long)(y0 - 1) + (long long)a.ny * (long long)(x0 - 1) : 0;
        }
        __syncwarp();  // converged for the warp-wide stores
        float *pix = spix + g * B2;
        const bool adu = a.adu;  // uniform over the launch
        // uniform over the launch as well
        const bool vec = ((reinterpret_cast<uintptr_t>(a.var) | reinterpret_cast<uintptr_t>(a.gain) |
                           reinterpret_cast<uintptr_t>(a.offset)) & 15u) == 0 && (a.ny & 3) == 0;
        if (vec) {
            const int sh = (int)(base & 3);
            const long long b0 = base - sh;
            float cb[16];  // the 16-column chunk being assembled for tensor memory
#pragma unroll
            for (int j = 0; j < BOX; j++) {
                const long long aj = b0 + (long long)a.ny * j;
                float v[BOX];
                map_column4<BOX>(a.var, aj, sh, ok, 0.f, v);
                if (adu) {
                    // a rejected or empty slot converts by (x - 0) * 1: unchanged
                    float o[BOX], gn[BOX];
                    map_column4<BOX>(a.offset, aj, sh, ok, 0.f, o);
                    map_column4<BOX>(a.gain, aj, sh, ok, 1.f, gn);
#pragma unroll
                    for (int i = 0; i < BOX; i++)
                        pix[BOX * j + i] = __fmul_rn(__fadd_rn(pix[BOX * j + i], -o[i]), gn[i]);
                }
#pragma unroll
                for (int i = 0; i < BOX; i++) {
                    const int p = BOX * j + i;
                    cb[p & 15] = v[i];
                    if ((p & 15) == 15) tmem_st16(taddr + (p & ~15), cb);
                }
            }
            if (B2 & 15) {  // the last, partial chunk: zeros past the tile
#pragma unroll
                for (int u = B2 & 15; u < 16; u++) cb[u] = 0.f;
                tmem_st16(taddr + (B2 & ~15), cb);
            }
        } else {
#pragma unroll
            for (int c = 0; c < TmemVar<BOX>::CHUNKS; c++) {
                float v[16], off[16], gn[16];
#pragma unroll
                for (int u = 0; u < 16; u++) {
                    const int p = 16 * c + u;
                    const int j = p / BOX, i = p - j * BOX;
                    const long long m = base + i + (long long)a.ny * j;
                    const bool in = ok && p < B2;
                    v[u] = in ? __ldg(a.var + m) : 0.f;
                    off[u] = (adu && in) ? __ldg(a.offset + m) : 0.f;
                    gn[u] = (adu && in) ? __ldg(a.gain + m) : 1.f;
                }
                tmem_st16(taddr + 16 * c, v);
                if (adu) {
                    // a rejected or empty slot converts by (x - 0) * 1: unchanged
#pragma unroll
                    for (int u = 0; u < 16; u++) {
                        const int p = 16 * c + u;
                        if (p < B2) pix[p] = __fmul_rn(__fadd_rn(pix[p], -off[u]), gn[u]);
                    }
                }
            }
        }
        tmem_wait_st();
        return ok;
    } else {
        static_assert(BOX <= 16, "two ROI columns per warp instruction");
        constexpr int NJP = (BOX + 1) / 2;  // column pairs of a ROI
        const int l = threadIdx.x & 31;
        const int r0 = threadIdx.x & ~31;  // the warp's first slot
        const int nw = min(max(nroi - r0, 0), 32);  // ROIs of this warp
        float *wpix = spix + r0 * B2;
        const float *src = a.data + (roi0 + r0) * B2;
        // this lane's place in a column pair: row i of column 2 jp + jj
        const int i = l & 15, jj = l >> 4;
        bool ok = l < nw;
        long long base = 0;
        if (ok) {
            const int32_t x0 = a.xc[roi0 + r0 + l], y0 = a.yc[roi0 + r0 + l];
            ok = x0 >= 1 && y0 >= 1 && x0 + BOX - 1 <= a.nx && y0 + BOX - 1 <= a.ny;
            if (!ok) atomicAdd(a.bad_corners, 1ull);
            base = ok ? (long long)(y0 - 1) + (long long)a.ny * (long long)(x0 - 1) : 0;
        }
        // variance tiles into the slots (zeros for rejected and empty slots)
        for (int r = 0; r < 32; r++) {
            const long long b = __shfl_sync(0xffffffffu, base, r);
            const bool okr = __shfl_sync(0xffffffffu, ok, r);
#pragma unroll
            for (int jp = 0; jp < NJP; jp++) {
                const int j = 2 * jp + jj;
                if (i < BOX && j < BOX)
                    cp_async4(wpix + r * B2 + j * BOX + i,
                              okr ? a.var + b + i + (long long)a.ny * j : a.var, okr ? 4u : 0u);
            }
        }
        cp_async_wait_all();
        __syncwarp();
#pragma unroll
        for (int c = 0; c < TmemVar<BOX>::CHUNKS; c++) {
            float v[16];
#pragma unroll
            for (int u = 0; u < 16; u++) {
                const int p = 16 * c + u;
                v[u] = p < B2 ? wpix[l * B2 + p] : 0.f;
            }
            tmem_st16(taddr + 16 * c, v);
        }
        tmem_wait_st();
        __syncwarp();  // every lane has read its slot
        // the warp's pixels over the slots
        const int cnt = nw * B2;
        if ((reinterpret_cast<uintptr_t>(src) & 15u) == 0) {
            const int c4 = cnt >> 2;
            for (int e = l; e < c4; e += 32) cp_async16(wpix + 4 * e, src + 4 * e);
            for (int e = (c4 << 2) + l; e < cnt; e += 32) cp_async4(wpix + e, src + e, 4);
        } else {
            for (int e = l; e < cnt; e += 32) cp_async4(wpix + e, src + e, 4);
        }
        for (int e = cnt + l; e < 32 * B2; e += 32) wpix[e] = 0.f;
        cp_async_wait_all();
        __syncwarp();
        // ADU -> e-, H ROIs (2 H NJP gathers of the maps) in flight at a time.
        // The conversion's dependent rounds of L2 gathers were 63 % of the
        // staging of a 15x15 block (clock64 per phase: 40.6 k of 64.7 k cycles;
        // staging 14 % of a block's life).  Measured, 300 000 ROIs: 15x15
        // with H = 4 1.824 -> 1.755 ms (H = 8: 1.808); 13x13 slower with more
        // (1.326 ms at H = 2, 1.344 at 4, 1.366 at 8): the fit's schedule
        // shifts with the registers the staging holds.
        if (a.adu) {
            constexpr int H = BOX >= 15 ? 4 : 2;
            for (int r = 0; r < nw; r += H) {
                float off[H][NJP], gn[H][NJP];
#pragma unroll
                for (int h = 0; h < H; h++) {
                    // lanes past the warp's ROIs hold ok == false
                    const long long b = __shfl_sync(0xffffffffu, base, (r + h) & 31);
                    const bool okr = __shfl_sync(0xffffffffu, ok, (r + h) & 31) && r + h < 32;
#pragma unroll
                    for (int jp = 0; jp < NJP; jp++) {
                        const int j = 2 * jp + jj;
                        off[h][jp] = 0.f;
                        gn[h][jp] = 1.f;
                        if (okr && i < BOX && j < BOX) {
                            const long long m = b + i + (long long)a.ny * j;
                            off[h][jp] = __ldg(a.offset + m);
                            gn[h][jp] = __ldg(a.gain + m);
                        }
                    }
                }
#pragma unroll
                for (int h = 0; h < H; h++) {
                    if (r + h >= nw) break;
#pragma unroll
                    for (int jp = 0; jp < NJP; jp++) {
                        const int j = 2 * jp + jj;
                        if (i < BOX && j < BOX) {
                            float *px = wpix + (r + h) * B2 + j * BOX + i;
                            *px = __fmul_rn(__fadd_rn(*px, -off[h][jp]), gn[h][jp]);
                        }
                    }
                }
            }
            __syncwarp();
        }
        return ok;
    }
}

// Stage the block's R ROIs (contiguous in global memory) into shared memory
// for the several-lanes-per-ROI kernel.  All pixel (and variance-tile) copies
// of a thread are issued as cp.async before any is waited for; for sCMOS the
// variance tile is gathered from the resident map and ADU data are converted,
// (ADU - offset) * gain (src/camera_models.jl:110-113), with the gain/offset
// loads batched.
template <int BOX, bool SCMOS>
__device__ __forceinline__ void stage_block(const KernelArgs &a, float *spix, int *sok, int R,
                                            int64_t roi0, int nroi)
{
    constexpr int B2 = BOX * BOX;
    constexpr int PS = SCMOS ? 2 : 1;  // floats per staged pixel
    long long *sbase = reinterpret_cast<long long *>(spix + R * B2 * PS);
    for (int g = threadIdx.x; g < R; g += blockDim.x) {
        int ok = g < nroi;
        long long base = 0;
        if (SCMOS && ok) {
            const int32_t x0 = a.xc[roi0 + g], y0 = a.yc[roi0 + g];
            ok = x0 >= 1 && y0 >= 1 && x0 + BOX - 1 <= a.nx && y0 + BOX - 1 <= a.ny;
            if (!ok) atomicAdd(a.bad_corners, 1ull);
            base = (long long)(y0 - 1) + (long long)a.ny * (long long)(x0 - 1);
        }
        sok[g] = ok;
        if (SCMOS) sbase[g] = base;
    }
    const float *src = a.data + roi0 * B2;
    const int cnt = nroi * B2;
    if (!SCMOS) {
        copy_data_plane<BOX>(spix, src, R, nroi);
    } else {
        __syncthreads();  // sok, sbase
        // consecutive e walk down a column: contiguous map addresses
        for (int e = threadIdx.x; e < R * B2; e += blockDim.x) {
            const int g = e / B2;
            const int p = e - g * B2, j = p / BOX, i = p - j * BOX;
            const bool in = e < cnt;
            const bool okg = in && sok[g];
            const long long m = sbase[g] + i + (long long)a.ny * j;
            cp_async4(spix + 2 * e, in ? src + e : a.data, in ? 4u : 0u);
            cp_async4(spix + 2 * e + 1, okg ? a.var + m : a.var, okg ? 4u : 0u);
        }
        cp_async_wait_all();
        if (a.adu) adu_to_electrons<BOX, 2>(a, spix, sok, sbase, cnt);
    }
    __syncthreads();
}

template <int MODEL> struct Slots {
    static constexpr int IX = 0, IY = 1;
    static constexpr int IN = (MODEL == 3) ? 3 : 2;
    static constexpr int IB = (MODEL == 3) ? 4 : 3;
};

// Likelihood terms of one pixel: compute_likelihood_terms, Poisson
// src/camera_models.jl:19-34 and sCMOS :36-42 (1/x by rcp_approx, 1 ulp).
template <bool SCMOS>
__device__ __forceinline__ void likelihood_terms(float d, float v, float mu, float &cf, float &df)
{
    if (!SCMOS) {
        const float rm = rcp_approx(mu);
        const float q = d * rm;
        const bool pos = mu > 0.01f;
        cf = pos ? fminf(q - 1.0f, 1e4f) : 0.f;
        df = pos ? fminf(q * rm, 1e4f) : 0.f;
    } else {
        const float rv = rcp_approx(mu + v);
        cf = (d - mu) * rv;
        df = rv;
    }
}

// Poisson terms where neither the mu > 0.01 test nor the 1e4 caps can act
// (uncapped() below): the same values without the tests.
__device__ __forceinline__ void likelihood_terms_uncapped(float d, float mu, float &cf, float &df)
{
    const float rm = rcp_approx(mu);
    const float q = d * rm;
    cf = q - 1.0f;
    df = q * rm;
}

// Whether a Poisson fit's pixel terms need no mu > 0.01 test and no 1e4 cap
// in this iteration: mu = fma(N psf_x, psf_y, bg) >= bg > 0.01 when N >= 0
// (psf >= 0 by construction), and with dmax the ROI's largest pixel,
// d / mu - 1 < d / bg <= 9900 and d / mu^2 <= d / bg^2 <= 9900 stay below the
// caps with room for the reciprocal's rounding.  NaN fails every test.
__device__ __forceinline__ bool uncapped(float N, float bg, float dmax)
{
    return bg > 0.01f && N >= 0.f && dmax <= 9900.f * fminf(bg, bg * bg);
}

// ---- two pixels at once: packed FP32 pairs ------------------------------------
//
// sm_100's add/mul/fma .f32x2 take one issue slot for two FP32 operations, each
// half rounded exactly like the scalar operation.  The one-thread kernel's
// Newton pixel loop runs rows (t, t+1) of a column as one pair.  Each half
// evaluates likelihood_terms / _uncapped's expressions with every operation
// rounded as written, none contracted into an FMA (d - mu as fma(mu, -1, d):
// one rounding, like the subtraction), as the reference evaluates them.
__device__ __forceinline__ float2 f2(float x) { return make_float2(x, x); }

template <bool SCMOS, bool UNCAPPED>
__device__ __forceinline__ void likelihood_terms2(float2 d, float2 v, float2 mu, float2 &cf,
                                                  float2 &df)
{
    if constexpr (SCMOS) {
        const float2 s = __fadd2_rn(mu, v);
        const float2 rv = make_float2(rcp_approx(s.x), rcp_approx(s.y));
        cf = __fmul2_rn(__ffma2_rn(mu, f2(-1.0f), d), rv);
        df = rv;
    } else {
        const float2 rm = make_float2(rcp_approx(mu.x), rcp_approx(mu.y));
        const float2 q = __fmul2_rn(d, rm);
        const float2 c = __fadd2_rn(q, f2(-1.0f));
        const float2 e = __fmul2_rn(q, rm);
        if constexpr (UNCAPPED) {
            cf = c;
            df = e;
        } else {
            const bool p0 = mu.x > 0.01f, p1 = mu.y > 0.01f;
            cf = make_float2(p0 ? fminf(c.x, 1e4f) : 0.f, p1 ? fminf(c.y, 1e4f) : 0.f);
            df = make_float2(p0 ? fminf(e.x, 1e4f) : 0.f, p1 ? fminf(e.y, 1e4f) : 0.f);
        }
    }
}

// Column-side contributions to gradient gs and diagonal Hessian hs of one pixel
// column j with x-table entry (xp, xd1, xd2, xs1, xs2) and the column sums
// A = sum_i py cf, B = sum_i py^2 df, E = sum_i cf, F = sum_i df,
// G = sum_i py ys1 df (dudt and d2udt2 as in src/psf_derivatives.jl).
template <int MODEL, int P>
__device__ __forceinline__ void col_terms(float (&gs)[P], float (&hs)[P], float xp, float xd1,
                                          float xd2, float xs1, float xs2, float A, float B,
                                          float E, float F, float Gc, const Axis &ax,
                                          const AstigWidths &aw)
{
    using S = Slots<MODEL>;
    gs[S::IX] = fmaf(xd1, A, gs[S::IX]);
    hs[S::IX] += xd2 * A - xd1 * xd1 * B;
    gs[S::IN] = fmaf(xp, A, gs[S::IN]);
    hs[S::IN] -= xp * xp * B;
    gs[S::IB] += E;
    hs[S::IB] -= F;
    if (MODEL == 1) {
        gs[4] = fmaf(xs1, A, gs[4]);
        hs[4] += (ax.m2s * xs1 - xs2) * A - xs1 * xs1 * B - 2.0f * xs1 * xp * Gc;
    } else if (MODEL == 2) {
        gs[4] = fmaf(xs1, A, gs[4]);
        hs[4] += (ax.m2s * xs1 - xs2) * A - xs1 * xs1 * B;
    } else if (MODEL == 3) {
        const float c1 = xs1 * aw.dsx;
        gs[2] = fmaf(c1, A, gs[2]);
        hs[2] += ((ax.m2s * xs1 - xs2) * (aw.dsx * aw.dsx) + xs1 * aw.d2sx) * A - c1 * c1 * B -
                 2.0f * c1 * (xp * aw.dsy) * Gc;
    }
}

// Row-side contributions of pixel row t: y-table entry (yd1, yd2, ys1, ys2) and
// the row sums C = sum_j xp cf, D = sum_j xp^2 df.
template <int MODEL, int P>
__device__ __forceinline__ void row_terms(float (&gs)[P], float (&hs)[P], float yd1, float yd2,
                                          float ys1, float ys2, float Ct, float Dt,
                                          const Axis &ay, const AstigWidths &aw)
{
    gs[1] = fmaf(yd1, Ct, gs[1]);
    hs[1] += yd2 * Ct - yd1 * yd1 * Dt;
    if (MODEL == 1) {
        gs[4] = fmaf(ys1, Ct, gs[4]);
        hs[4] += (ay.m2s * ys1 - ys2) * Ct - ys1 * ys1 * Dt;
    } else if (MODEL == 2) {
        gs[5] = fmaf(ys1, Ct, gs[5]);
        hs[5] += (ay.m2s * ys1 - ys2) * Ct - ys1 * ys1 * Dt;
    } else if (MODEL == 3) {
        const float c2 = ys1 * aw.dsy;
        gs[2] = fmaf(c2, Ct, gs[2]);
        hs[2] += ((ay.m2s * ys1 - ys2) * (aw.dsy * aw.dsy) + ys1 * aw.d2sy) * Ct - c2 * c2 * Dt;
    }
}

// Scalar Newton step, src/unified_kernel.jl:337-350, with apply_constraints!,
// src/constraints.jl:49-53.
template <int P>
__device__ __forceinline__ void newton_step(float (&th)[P], const float (&gs)[P],
                                            const float (&hs)[P], const KernelArgs &a)
{
#pragma unroll
    for (int k = 0; k < P; k++) {
        const float delta = fabsf(hs[k]) > 1e-10f ? __fdiv_rn(gs[k], hs[k]) : 0.f;
        const float step = jl_clamp(delta, -a.max_step[k], a.max_step[k]);
        th[k] = jl_clamp(__fadd_rn(th[k], -step), a.lower[k], a.upper[k]);
    }
}

// Separable structure of dudt_k = sum_t a_kt(j) * b_kt(i): each parameter has
// one or two terms, each a column function a (x-axis tables) times a row
// function b, with b in {0: psf_y, 1: d psf_y/dy, 2: 1, 3: d psf_y/dsigma_y}.
__host__ __device__ constexpr int term_count(int model, int k)
{
    return ((model == 1 && k == 4) || (model == 3 && k == 2)) ? 2 : 1;
}
__host__ __device__ constexpr int term_b(int model, int k, int t)
{
    // parameter slots: x 0, y 1; N, bg at 2, 3 (3, 4 for the astigmatic model)
    return model == 3 ? (k == 0 ? 0 : k == 1 ? 1 : k == 2 ? (t == 0 ? 0 : 3) : k == 3 ? 0 : 2)
                      : (k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 0 : k == 3 ? 2
                                                   : k == 4 ? (model == 1 ? (t == 0 ? 0 : 3) : 0)
                                                            : 3);
}

template <int NB>
__device__ __forceinline__ float qsym(const float (&Q)[NB][NB], int p, int q)
{
    return p <= q ? Q[p][q] : Q[q][p];
}

// Per pixel of the final pass: the LLR term (compute_log_likelihood,
// src/camera_models.jl:60-96) and the Fisher weight sums Q_pq += b_p b_q w,
// w = 1/variance over pixels with mu > 0 (src/unified_kernel.jl:378-396).
// FAST_LOG: the Poisson LLR's logarithms by log_approx (the final pass, whose
// LLR is an output only); the full-Hessian passes, which accept or reject a
// step on the LLR, keep the library's logf.
template <bool SCMOS, bool SIG, int NB, bool FAST_LOG = true>
__device__ __forceinline__ void final_pixel(float d, float v, float mu, float py, float yd1,
                                            float ys1, float &llr, float (&Q)[NB][NB])
{
    const float rv = rcp_approx(SCMOS ? mu + v : mu);
    if (!SCMOS) {
        if (mu > 0.f && d > 0.f) {
            const float lm = FAST_LOG ? log_approx(mu) : logf(mu);
            const float ld = FAST_LOG ? log_approx(d) : logf(d);
            llr += d * lm - mu - (d * ld - d);
        } else if (mu > 0.f && d == 0.f) {
            llr -= mu;
        }
    } else {
        const float tv = mu + v;
        if (tv > 0.f) {
            const float res = d - mu;
            llr += -0.5f * ((res * res) * rv);
        }
    }
    const float w = mu > 0.f ? rv : 0.f;
    const float t0 = py * w, t1 = yd1 * w;
    Q[0][0] = fmaf(t0, py, Q[0][0]);
    Q[0][1] = fmaf(t0, yd1, Q[0][1]);
    Q[0][2] += t0;
    Q[1][1] = fmaf(t1, yd1, Q[1][1]);
    Q[1][2] += t1;
    Q[2][2] += w;
    if (SIG) {
        const float t3 = ys1 * w;
        Q[0][3] = fmaf(t0, ys1, Q[0][3]);
        Q[1][3] = fmaf(t1, ys1, Q[1][3]);
        Q[2][3] += t3;
        Q[3][3] = fmaf(t3, ys1, Q[3][3]);
    }
}

// One column's Fisher contribution: F_kl += sum_{t,u} a_kt a_lu Q[b_kt][b_lu],
// summed in FP32 for the column and accumulated across columns as a
// double-float (Fh + Fl, upper triangle).
template <int MODEL, int P, int NB>
__device__ __forceinline__ void fisher_column(float (&Fh)[P][P], float (&Fl)[P][P],
                                              const float (&Q)[NB][NB], float xp, float xd1,
                                              float xs1, const AstigWidths &aw)
{
    using S = Slots<MODEL>;
    float av[P][2];
    av[S::IX][0] = xd1; av[S::IX][1] = 0.f;
    av[S::IY][0] = xp;  av[S::IY][1] = 0.f;
    av[S::IN][0] = xp;  av[S::IN][1] = 0.f;
    av[S::IB][0] = 1.f; av[S::IB][1] = 0.f;
    if (MODEL == 1) { av[4][0] = xs1; av[4][1] = xp; }
    if (MODEL == 2) { av[4][0] = xs1; av[4][1] = 0.f; av[5][0] = xp; av[5][1] = 0.f; }
    if (MODEL == 3) { av[2][0] = xs1 * aw.dsx; av[2][1] = xp * aw.dsy; }
#pragma unroll
    for (int k = 0; k < P; k++)
#pragma unroll
        for (int l = k; l < P; l++) {
            float s = 0.f;
#pragma unroll
            for (int tk = 0; tk < term_count(MODEL, k); tk++)
#pragma unroll
                for (int tl = 0; tl < term_count(MODEL, l); tl++)
                    s = fmaf(av[k][tk] * av[l][tl],
                             qsym<NB>(Q, term_b(MODEL, k, tk), term_b(MODEL, l, tl)), s);
            dd_add(Fh[k][l], Fl[k][l], s);
        }
}

// ---- full-Hessian method (GMLE_METHOD_FISHER_LM; no reference counterpart) ----
//
// An option beside the reference's per-parameter Newton step: each pass at
// a candidate theta gives the log-likelihood L (compute_log_likelihood,
// src/camera_models.jl:60-96), the gradient g_k = sum dudt_k cf (the
// reference's likelihood terms, src/camera_models.jl:19-42) and the expected
// information F_kl = sum dudt_k dudt_l / v over mu > 0 (the Fisher matrix of
// src/unified_kernel.jl:378-396).  A candidate at least as likely as the best
// so far (to 1e-5 |L|, the rounding of an FP32 sum of up to 225 terms, so that
// near the maximum the decision does not turn on rounding) is accepted, with
// its g and F, and the damping lambda falls tenfold; a worse one is rejected
// and lambda rises tenfold.  The next step
// solves (F + lambda diag F) step = g at the best point (Fisher scoring with
// Levenberg-Marquardt damping), clamped like the reference's steps
// (max_step, then the bounds).  The final pass is the reference's, at the
// best point.

// Per pixel of a full-Hessian pass: final_pixel's LLR and Fisher weight
// sums, plus the gradient's row sums R_b += b cf.
template <bool SCMOS, bool SIG, int NB>
__device__ __forceinline__ void lm_pixel(float d, float v, float mu, float py, float yd1,
                                         float ys1, float &llr, float (&Q)[NB][NB],
                                         float (&Rs)[NB])
{
    final_pixel<SCMOS, SIG, NB, false>(d, v, mu, py, yd1, ys1, llr, Q);
    float cf, df;
    likelihood_terms<SCMOS>(d, v, mu, cf, df);
    Rs[0] = fmaf(py, cf, Rs[0]);
    Rs[1] = fmaf(yd1, cf, Rs[1]);
    Rs[2] += cf;
    if (SIG) Rs[3] = fmaf(ys1, cf, Rs[3]);
}

// One column's contribution to F (upper triangle) and g, in FP32.
template <int MODEL, int P, int NB>
__device__ __forceinline__ void lm_column(float (&F)[P][P], float (&g)[P], const float (&Q)[NB][NB],
                                          const float (&Rs)[NB], float xp, float xd1, float xs1,
                                          const AstigWidths &aw)
{
    using S = Slots<MODEL>;
    float av[P][2];
    av[S::IX][0] = xd1; av[S::IX][1] = 0.f;
    av[S::IY][0] = xp;  av[S::IY][1] = 0.f;
    av[S::IN][0] = xp;  av[S::IN][1] = 0.f;
    av[S::IB][0] = 1.f; av[S::IB][1] = 0.f;
    if (MODEL == 1) { av[4][0] = xs1; av[4][1] = xp; }
    if (MODEL == 2) { av[4][0] = xs1; av[4][1] = 0.f; av[5][0] = xp; av[5][1] = 0.f; }
    if (MODEL == 3) { av[2][0] = xs1 * aw.dsx; av[2][1] = xp * aw.dsy; }
#pragma unroll
    for (int k = 0; k < P; k++) {
#pragma unroll
        for (int tk = 0; tk < term_count(MODEL, k); tk++)
            g[k] = fmaf(av[k][tk], Rs[term_b(MODEL, k, tk)], g[k]);
#pragma unroll
        for (int l = k; l < P; l++) {
            float sum = 0.f;
#pragma unroll
            for (int tk = 0; tk < term_count(MODEL, k); tk++)
#pragma unroll
                for (int tl = 0; tl < term_count(MODEL, l); tl++)
                    sum = fmaf(av[k][tk] * av[l][tl],
                               qsym<NB>(Q, term_b(MODEL, k, tk), term_b(MODEL, l, tl)), sum);
            F[k][l] += sum;
        }
    }
}

// Accept or reject the pass's candidate th (log-likelihood L, gradient g,
// information F, upper triangle) against the best point thb (Lb, gb, Fb),
// then the next step from the best point into stp.
template <int P>
__device__ __forceinline__ void lm_update(const float (&th)[P], float (&thb)[P], float (&stp)[P],
                                          float (&gb)[P], float (&Fb)[P][P], float &Lb,
                                          float &lam, bool first, float L, const float (&g)[P],
                                          const float (&F)[P][P])
{
    if (first || L >= Lb - 1e-5f * fabsf(Lb)) {
#pragma unroll
        for (int k = 0; k < P; k++) {
            thb[k] = th[k];
            gb[k] = g[k];
#pragma unroll
            for (int l = k; l < P; l++) Fb[k][l] = F[k][l];
        }
        Lb = L;
        lam = fmaxf(lam * 0.1f, 1e-7f);
    } else {
        lam = fminf(lam * 10.f, 1e7f);
    }
    // Cholesky of A = Fb + lam diag(Fb) (lower factor Lm), then two solves
    float Lm[P][P], y[P];
    bool ok = true;
#pragma unroll
    for (int j = 0; j < P; j++) {
        float sd = Fb[j][j] + lam * Fb[j][j];
#pragma unroll
        for (int k = 0; k < j; k++) sd -= Lm[j][k] * Lm[j][k];
        ok = ok && sd > 0.f;
        const float dj = sqrtf(fmaxf(sd, 1e-30f));
        Lm[j][j] = dj;
#pragma unroll
        for (int i = j + 1; i < P; i++) {
            float si = Fb[j][i];
#pragma unroll
            for (int k = 0; k < j; k++) si -= Lm[i][k] * Lm[j][k];
            Lm[i][j] = __fdiv_rn(si, dj);
        }
    }
#pragma unroll
    for (int i = 0; i < P; i++) {
        float si = gb[i];
#pragma unroll
        for (int k = 0; k < i; k++) si -= Lm[i][k] * y[k];
        y[i] = __fdiv_rn(si, Lm[i][i]);
    }
#pragma unroll
    for (int i = P - 1; i >= 0; i--) {
        float si = y[i];
#pragma unroll
        for (int k = i + 1; k < P; k++) si -= Lm[k][i] * stp[k];
        stp[i] = __fdiv_rn(si, Lm[i][i]);
    }
    if (!ok) {  // not positive definite: the diagonal step
#pragma unroll
        for (int k = 0; k < P; k++) stp[k] = Fb[k][k] > 0.f ? __fdiv_rn(gb[k], Fb[k][k]) : 0.f;
    }
}

template <int P>
__device__ __forceinline__ void write_result(const KernelArgs &a, int64_t roi, bool valid,
                                             const float (&th)[P], double (&Fm)[P][P], float llr)
{
    if (valid) {
        float cr[P];
        const uint8_t fl = crlb_from_fisher<P>(Fm, cr);
#pragma unroll
        for (int k = 0; k < P; k++) {
            a.params[roi * P + k] = th[k];
            a.crlb[roi * P + k] = cr[k];
        }
        a.llr[roi] = llr;
        if (a.flags) a.flags[roi] = fl;
    } else {
        // corner outside the calibration map: no fit
        const float qnan = __int_as_float(0x7fc00000);
#pragma unroll
        for (int k = 0; k < P; k++) { a.params[roi * P + k] = qnan; a.crlb[roi * P + k] = qnan; }
        a.llr[roi] = qnan;
        if (a.flags) a.flags[roi] = 0;
    }
}

// The results of a warp's 32 consecutive ROIs (one per lane), written as
// contiguous runs.  Each lane's parameters, then its CRLBs, go through the
// warp's own stage of 32 P floats in shared memory (the pixel slots of its
// ROIs, whose fits are done), so that a warp store writes 32 consecutive
// words instead of 32 words P floats apart.  Outputs in the caller's pinned
// host memory are written over the host link, where scattered 4-byte writes
// are separate transactions that slow every transfer sharing the link (the
// serving loop's input copies among them).  g = this lane's slot, nroi = the
// block's ROIs from roi0; every lane of the warp calls it.
template <int P>
__device__ __forceinline__ void write_results_warp(const KernelArgs &a, int64_t roi0, int g,
                                                   int nroi, bool valid, const float (&th)[P],
                                                   double (&Fm)[P][P], float llr, float *stage)
{
    const float qnan = __int_as_float(0x7fc00000);
    float cr[P], tv[P];
    uint8_t fl = 0;
    if (valid && g < nroi) {
        fl = crlb_from_fisher<P>(Fm, cr);
#pragma unroll
        for (int k = 0; k < P; k++) tv[k] = th[k];
    } else {
        // corner outside the calibration map (or an empty slot): no fit
#pragma unroll
        for (int k = 0; k < P; k++) { cr[k] = qnan; tv[k] = qnan; }
        llr = qnan;
    }
    const int lane = threadIdx.x & 31;
    const int w0 = g - lane;                     // the warp's first slot
    const int nw = min(max(nroi - w0, 0), 32);   // its ROIs
    const int64_t base = (roi0 + w0) * P;
#pragma unroll
    for (int pass = 0; pass < 2; pass++) {
        __syncwarp();  // the stage is free (pixels read, or the previous pass written)
#pragma unroll
        for (int k = 0; k < P; k++) stage[lane * P + k] = pass ? cr[k] : tv[k];
        __syncwarp();
        float *out = pass ? a.crlb : a.params;
        for (int e = lane; e < nw * P; e += 32) out[base + e] = stage[e];
    }
    if (g < nroi) {
        a.llr[roi0 + g] = llr;
        if (a.flags) a.flags[roi0 + g] = fl;
    }
}

template <int MODEL>
__device__ __forceinline__ void axis_widths(const float *th, const KernelArgs &a, float &sxw,
                                            float &syw, AstigWidths &aw)
{
    if (MODEL == 0) { sxw = syw = a.psf[0]; }
    else if (MODEL == 1) { sxw = syw = th[4]; }
    else if (MODEL == 2) { sxw = th[4]; syw = th[5]; }
    else { astig_widths(th[2], a.psf, aw); sxw = aw.sx; syw = aw.sy; }
}

// ---- kernel 1: one thread per ROI ---------------------------------------------
//
// Each thread fits one ROI with every axis table in registers; per column the
// next column's erf/exp evaluations are issued before the current column's
// pixel work so that their latency overlaps it.  Occupancy is bounded by
// shared memory (the staged pixels), so registers are not the constraint.
//
// fit_rois_r1 fits ROIs [roi0, roi0 + nroi) of `a` (nroi <= blockDim.x) with
// the block's threads, staging them in `smem`; the plain kernel calls it once
// per block, the persistent mixed-batch kernel once per work tile.
template <int MODEL, int BOX, bool SCMOS, bool LM = false>
__device__ __forceinline__ void fit_rois_r1(const KernelArgs &a, int64_t roi0, int nroi,
                                            float *smem, uint32_t taddr)
{
    constexpr int P = ModelInfo<MODEL>::P;
    constexpr bool SIG = ModelInfo<MODEL>::SIG;
    constexpr bool CROSS = (MODEL == 1 || MODEL == 3);
    constexpr int B2 = BOX * BOX;
    constexpr int PS = 1;  // data plane; sCMOS variance tiles are in tensor memory
    constexpr int NB = SIG ? 4 : 3;
    constexpr int LW = TmemVar<BOX>::LW;
    // edge walks with the warp-voted erf re-evaluation (walk_entry)
    constexpr bool VOTE = SCMOS && ((MODEL == 3 && BOX >= 15) || BOX <= 7);
    using S = Slots<MODEL>;
    static_assert(B2 >= P, "a warp's pixel slots stage its results");

    float *spix = smem;
    const bool valid = stage_r1<BOX, SCMOS>(a, spix, roi0, nroi, taddr);

    const int g = threadIdx.x;
    if (__all_sync(0xffffffffu, g >= nroi)) return;
    const float *pix = spix + g * B2 * PS;

    float th[P];
#pragma unroll
    for (int k = 0; k < P; k++) th[k] = 0.f;
    initialize<MODEL, BOX, PS>(pix, a.psf, th);
    // Poisson: the ROI's largest pixel (NaN if any pixel is NaN), for uncapped()
    float dmax = 0.f;
    if (!SCMOS && !LM) {
        dmax = -INFINITY;
        for (int p = 0; p < B2; p++) {
            const float d = pix[p];
            dmax = (d > dmax || d != d) ? d : dmax;
        }
    }

    float py[BOX], yd1[BOX], yd2[BOX], ys1[SIG ? BOX : 1], ys2[SIG ? BOX : 1];
    // full-Hessian method: best point, its log-likelihood, next step, damping
    constexpr int PL = LM ? P : 1;
    float thb[PL], stp[PL], gb[PL], Fb[PL][PL], Lb = -INFINITY, lam = 1e-3f;
#pragma unroll
    for (int k = 0; k < PL; k++) { thb[k] = th[k]; stp[k] = 0.f; }
    for (int it = 0; it <= a.iterations; ++it) {
        const bool final_pass = (it == a.iterations);
        if (LM && it > 0) {
#pragma unroll
            for (int k = 0; k < PL; k++)
                th[k] = final_pass ? thb[k]
                                   : jl_clamp(__fadd_rn(thb[k], jl_clamp(stp[k], -a.max_step[k],
                                                                         a.max_step[k])),
                                              a.lower[k], a.upper[k]);
        }
        float sxw, syw;
        AstigWidths aw;
        axis_widths<MODEL>(th, a, sxw, syw, aw);
        const float N = th[S::IN], bg = th[S::IB];
        const Axis ax = make_axis(th[S::IX], sxw, N, a.sqrt2pi, SIG);
        const Axis ay = make_axis(th[S::IY], syw, N, a.sqrt2pi, SIG);
        {
            EdgeWalk wy = walk_start(1, ay);
#pragma unroll
            for (int t = 0; t < BOX; t++) {
                float s1 = 0.f, s2 = 0.f;
                walk_entry<SIG, true, VOTE>(t + 1, ay, wy, py[t], yd1[t], yd2[t], s1, s2);
                if (SIG) { ys1[t] = s1; ys2[t] = s2; }
            }
        }
        EdgeWalk wx = walk_start(1, ax);
        float xp, xd1, xd2, xs1 = 0.f, xs2 = 0.f;
        walk_entry<SIG, true, VOTE>(1, ax, wx, xp, xd1, xd2, xs1, xs2);

        if (LM && !final_pass) {
            float llr = 0.f;
            float F[P][P], gs[P];
#pragma unroll
            for (int k = 0; k < P; k++) {
                gs[k] = 0.f;
#pragma unroll
                for (int l = 0; l < P; l++) F[k][l] = 0.f;
            }
            for (int j = 1; j <= BOX; j++) {
                float nxp, nxd1, nxd2, nxs1 = 0.f, nxs2 = 0.f;
                walk_entry<SIG, false, VOTE>(j + 1, ax, wx, nxp, nxd1, nxd2, nxs1, nxs2);
                const float npx = N * xp;
                const float *col = pix + (j - 1) * BOX * PS;
                float vv[LW];  // this column's variances, from tensor memory
                if (SCMOS) tmem_ld<LW>(taddr + BOX * (j - 1), vv);
                float Q[NB][NB], Rs[NB];
#pragma unroll
                for (int p = 0; p < NB; p++) {
                    Rs[p] = 0.f;
#pragma unroll
                    for (int q = 0; q < NB; q++) Q[p][q] = 0.f;
                }
#pragma unroll
                for (int t = 0; t < BOX; t++) {
                    const float d = col[t];
                    const float v = SCMOS ? vv[t] : 0.f;
                    const float mu = fmaf(npx, py[t], bg);
                    lm_pixel<SCMOS, SIG, NB>(d, v, mu, py[t], yd1[t], SIG ? ys1[t] : 0.f, llr, Q,
                                             Rs);
                }
                lm_column<MODEL, P, NB>(F, gs, Q, Rs, xp, xd1, xs1, aw);
                xp = nxp; xd1 = nxd1; xs1 = nxs1;
            }
            if constexpr (LM) lm_update<P>(th, thb, stp, gb, Fb, Lb, lam, it == 0, llr, gs, F);
        } else if (!final_pass) {
            // rows (2k, 2k + 1) as packed pairs (likelihood_terms2); an odd
            // box's last row (even: the first partial sums) runs alone
            constexpr int NPR = BOX / 2;
            constexpr bool ODD = (BOX & 1) != 0;
            float2 pyP[NPR], py2P[NPR], aGP[CROSS ? NPR : 1], CP[NPR], DP[NPR];
#pragma unroll
            for (int k = 0; k < NPR; k++) {
                pyP[k] = make_float2(py[2 * k], py[2 * k + 1]);
                py2P[k] = __fmul2_rn(pyP[k], pyP[k]);
                if (CROSS) aGP[k] = make_float2(py[2 * k] * ys1[2 * k],
                                                py[2 * k + 1] * ys1[2 * k + 1]);
                CP[k] = f2(0.f);
                DP[k] = f2(0.f);
            }
            const float pyl = py[BOX - 1], py2l = pyl * pyl;
            const float aGl = CROSS ? pyl * ys1[BOX - 1] : 0.f;
            float Cl = 0.f, Dl = 0.f;
            const float2 Nv = f2(N), bgv = f2(bg);
            float gs[P], hs[P];
#pragma unroll
            for (int k = 0; k < P; k++) { gs[k] = 0.f; hs[k] = 0.f; }
            // this column's variances from tensor memory.  For 15x15 (two
            // blocks of 4 warps per SM, whatever its registers) the next
            // column's load is issued before this column's pixel work and
            // waited for after it: measured 2.31 -> 2.22 ms for 300 000
            // astigmatic ROIs.  The smaller boxes hide the load with their
            // warps (13x13 measured slightly slower pipelined) and keep their
            // registers.
            constexpr bool PIPE = SCMOS && BOX >= 15;
            float vv[LW];
            if (PIPE) tmem_ld<LW>(taddr, vv);
            // the column loop, with (UNCAPPED) or without the Poisson terms'
            // tests and caps
            auto columns = [&](auto uncapped_tag) {
                constexpr bool UNCAPPED = decltype(uncapped_tag)::value;
                for (int j = 1; j <= BOX; j++) {
                    // next column's table entry: independent of this column's pixels
                    float nxp, nxd1, nxd2, nxs1 = 0.f, nxs2 = 0.f;
                    walk_entry<SIG, true, VOTE>(j + 1, ax, wx, nxp, nxd1, nxd2, nxs1, nxs2);
                    const float2 xpv = f2(xp);
                    const float2 npx = __fmul2_rn(Nv, xpv), xp2 = __fmul2_rn(xpv, xpv);
                    const float *col = pix + (j - 1) * BOX * PS;
                    float nv[LW];
                    if (PIPE && j < BOX) tmem_ld_start<LW>(taddr + BOX * j, nv);
                    if (SCMOS && !PIPE) tmem_ld<LW>(taddr + BOX * (j - 1), vv);
                    // even and odd rows in separate partial sums (.x, .y): two
                    // independent FMA chains of box/2 instead of one of box
                    float2 A = f2(0.f), B = f2(0.f), E = f2(0.f), F = f2(0.f), Gc = f2(0.f);
#pragma unroll
                    for (int k = 0; k < NPR; k++) {
                        const int t = 2 * k;
                        const float2 d = make_float2(col[t], col[t + 1]);
                        const float2 v = SCMOS ? make_float2(vv[t], vv[t + 1]) : f2(0.f);
                        const float2 mu = __ffma2_rn(npx, pyP[k], bgv);
                        float2 cf, df;
                        likelihood_terms2<SCMOS, UNCAPPED>(d, v, mu, cf, df);
                        A = __ffma2_rn(pyP[k], cf, A);
                        B = __ffma2_rn(py2P[k], df, B);
                        E = __fadd2_rn(E, cf);
                        F = __fadd2_rn(F, df);
                        CP[k] = __ffma2_rn(xpv, cf, CP[k]);
                        DP[k] = __ffma2_rn(xp2, df, DP[k]);
                        if (CROSS) Gc = __ffma2_rn(aGP[k], df, Gc);
                    }
                    if constexpr (ODD) {
                        const float d = col[BOX - 1];
                        const float v = SCMOS ? vv[BOX - 1] : 0.f;
                        const float mu = fmaf(npx.x, pyl, bg);
                        float cf, df;
                        if constexpr (UNCAPPED) likelihood_terms_uncapped(d, mu, cf, df);
                        else likelihood_terms<SCMOS>(d, v, mu, cf, df);
                        A.x = fmaf(pyl, cf, A.x);
                        B.x = fmaf(py2l, df, B.x);
                        E.x += cf;
                        F.x += df;
                        Cl = fmaf(xp, cf, Cl);
                        Dl = fmaf(xp2.x, df, Dl);
                        if (CROSS) Gc.x = fmaf(aGl, df, Gc.x);
                    }
                    col_terms<MODEL, P>(gs, hs, xp, xd1, xd2, xs1, xs2, A.x + A.y, B.x + B.y,
                                        E.x + E.y, F.x + F.y, Gc.x + Gc.y, ax, aw);
                    if (PIPE && j < BOX) {
                        tmem_ld_wait<LW>(nv);
#pragma unroll
                        for (int q = 0; q < LW; q++) vv[q] = nv[q];
                    }
                    xp = nxp; xd1 = nxd1; xd2 = nxd2; xs1 = nxs1; xs2 = nxs2;
                }
            };
            if constexpr (!SCMOS) {
                // one decision per warp (empty slots do not hold it back)
                if (__all_sync(0xffffffffu, g >= nroi || uncapped(N, bg, dmax)))
                    columns(std::true_type{});
                else
                    columns(std::false_type{});
            } else {
                columns(std::false_type{});
            }
#pragma unroll
            for (int t = 0; t < BOX; t++) {
                const bool pr = t < 2 * NPR;
                const float Ct = pr ? ((t & 1) ? CP[t >> 1].y : CP[t >> 1].x) : Cl;
                const float Dt = pr ? ((t & 1) ? DP[t >> 1].y : DP[t >> 1].x) : Dl;
                row_terms<MODEL, P>(gs, hs, yd1[t], yd2[t], SIG ? ys1[t] : 0.f,
                                    SIG ? ys2[t] : 0.f, Ct, Dt, ay, aw);
            }
            newton_step<P>(th, gs, hs, a);
        } else {
            float llr = 0.f;
            float Fh[P][P], Fl[P][P];
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = 0; l < P; l++) { Fh[k][l] = 0.f; Fl[k][l] = 0.f; }
            for (int j = 1; j <= BOX; j++) {
                float nxp, nxd1, nxd2, nxs1 = 0.f, nxs2 = 0.f;
                walk_entry<SIG, false, VOTE>(j + 1, ax, wx, nxp, nxd1, nxd2, nxs1, nxs2);
                const float npx = N * xp;
                const float *col = pix + (j - 1) * BOX * PS;
                float vv[LW];  // this column's variances, from tensor memory
                if (SCMOS) tmem_ld<LW>(taddr + BOX * (j - 1), vv);
                float Q[NB][NB];
#pragma unroll
                for (int p = 0; p < NB; p++)
#pragma unroll
                    for (int q = 0; q < NB; q++) Q[p][q] = 0.f;
#pragma unroll
                for (int t = 0; t < BOX; t++) {
                    const float d = col[t];
                    const float v = SCMOS ? vv[t] : 0.f;
                    const float mu = fmaf(npx, py[t], bg);
                    final_pixel<SCMOS, SIG, NB>(d, v, mu, py[t], yd1[t], SIG ? ys1[t] : 0.f, llr, Q);
                }
                fisher_column<MODEL, P, NB>(Fh, Fl, Q, xp, xd1, xs1, aw);
                xp = nxp; xd1 = nxd1; xs1 = nxs1;
            }
            double Fm[P][P];
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = k; l < P; l++) {
                    Fm[k][l] = dd_to_double(Fh[k][l], Fl[k][l]);
                    Fm[l][k] = Fm[k][l];
                }
            // the warp's pixel slots (32 box^2 >= 32 P floats) stage its results
            write_results_warp<P>(a, roi0, g, nroi, valid, th, Fm, llr,
                                  spix + (size_t)(threadIdx.x & ~31) * B2);
        }
    }
}

// TABLE = false: plain launch, block b fits ROIs [b R, b R + R) of `a` (the
// kernel parameter, read from the constant bank).  TABLE = true: table launch
// (`a` supplies only tpr); the block fits tiles of the table's groups, each
// through the block's shared-memory copy of the tile's group arguments, until
// none is left.
//
// sCMOS: warp 0 allocates the CTA's tensor memory for the variance tiles before
// the first tile and frees it after the last; no path leaves the kernel
// between the two.
//
// Residency: no minimum of blocks per SM (an explicit 1 lets the compiler
// take up to 255 registers: XYNB 11x11 sCMOS 251 instead of 142, two blocks
// per SM instead of three).  XYNBS 9x9 sCMOS measured 0.962 ms for 500 000
// ROIs when held to 128 registers for a fourth block (with 52 bytes of
// spills), 0.952 ms with its own 164 registers and three blocks.
template <int MODEL, int BOX, bool SCMOS, bool TABLE, bool LM = false>
__global__ void __launch_bounds__(128)
    fit_kernel_r1(const KernelArgs a, const TileTable t)
{
    extern __shared__ __align__(16) float smem[];
    __shared__ uint32_t s_tmem;
    constexpr int NCOLS = TmemVar<BOX>::NCOLS;
    const int R = blockDim.x;
    uint32_t taddr = 0;
    if (SCMOS) {
        if (threadIdx.x < 32) tmem_alloc<NCOLS>(&s_tmem);
        tmem_sync();
        taddr = s_tmem + ((uint32_t)(((threadIdx.x >> 5) & 3) * 32) << 16);
    }
    if (!TABLE) {
        const int64_t roi0 = (int64_t)blockIdx.x * R;
        const int64_t left = a.n - roi0;
        fit_rois_r1<MODEL, BOX, SCMOS, LM>(a, roi0, left < R ? (int)left : R, smem, taddr);
    } else {
        TableSlot *ts = table_slot(smem, smem_bytes(MODEL, BOX, SCMOS, 1, R));
        table_slot_init(ts);
        int64_t roi0;
        int nroi;
        for (int k = 0; table_next(t, R, ts, k, roi0, nroi); k++) {
            fit_rois_r1<MODEL, BOX, SCMOS>(ts->a, roi0, nroi, smem, taddr);
            __syncthreads();  // the tile's shared memory and slot are free again
        }
    }
    if (SCMOS) {
        tmem_sync();  // every warp's tensor-memory loads have completed
        if (threadIdx.x < 32) tmem_dealloc<NCOLS>(s_tmem);
    }
}

// ---- kernel 2: several threads per ROI ------------------------------------------
//
// For batches too small to fill the GPU with one thread per ROI.  TPR lanes
// (2, 4 or 8) of one warp share a ROI as a grid of NCX column blocks by NRY row
// blocks (2 x 1, 4 x 1, 4 x 2): lane (rx, ry) owns columns
// [rx BOX / NCX, (rx + 1) BOX / NCX) and rows [ry BOX / NRY, (ry + 1) BOX / NRY)
// of the ROI, evaluates the edge tables of its own columns and rows only, and
// sums its own pixels.  The column and row terms of the gradient and Hessian
// (col_terms, row_terms) and the Fisher column terms (fisher_column) are
// linear in the per-column and per-row sums, so each lane applies them to its
// partial sums, and only the 2P gradient and Hessian values (and, once, the
// Fisher matrix and the log-likelihood) are combined across the lanes, by
// warp shuffles.  Every lane then takes the same Newton step, so theta stays
// identical in all of them.  The initial estimate is computed by every lane
// from the staged ROI, in the reference's order.  As in the one-thread
// kernel, the next column's table entry is evaluated ahead of the current
// column's pixels, and whole columns of rows are independent work: a lane
// alone on its scheduler is bound by these chains' latency, not by issue.
//
// Two column blocks evaluate only the y tables twice; four lanes cut a lane's
// instructions further but add 79 % to the ROI's total (10 000 XYNB 11x11
// ROIs: 127 k against 71 k lane instructions per ROI).  Measured at 10 000
// ROIs: astigmatic 15x15 sCMOS 157 us with two lanes, 234 us with four; XYNB
// 11x11 Poisson 77, 72 and 73 us with two, four and one, where a fit is
// bound by the latency of its 21 dependent passes.
template <int TPR> struct LaneGrid {
    static_assert(TPR == 2 || TPR == 4 || TPR == 8, "2, 4 or 8 lanes per ROI");
    static constexpr int NCX = TPR == 2 ? 2 : 4;
    static constexpr int NRY = TPR / NCX;
};

// fit_rois_tpr fits ROIs [roi0, roi0 + nroi) of `a` (nroi <= blockDim.x / TPR).
template <int MODEL, int BOX, bool SCMOS, int TPR>
__device__ __forceinline__ void fit_rois_tpr(const KernelArgs &a, int64_t roi0, int nroi,
                                             float *smem)
{
    constexpr int P = ModelInfo<MODEL>::P;
    constexpr bool SIG = ModelInfo<MODEL>::SIG;
    constexpr bool CROSS = (MODEL == 1 || MODEL == 3);
    constexpr int B2 = BOX * BOX;
    constexpr int PS = SCMOS ? 2 : 1;
    constexpr int NB = SIG ? 4 : 3;
    constexpr int NCX = LaneGrid<TPR>::NCX, NRY = LaneGrid<TPR>::NRY;
    constexpr int RMAX = (BOX + NRY - 1) / NRY;  // rows of the largest row block
    using S = Slots<MODEL>;

    const int R = blockDim.x / TPR;
    float *spix = smem;
    int *sok = reinterpret_cast<int *>(spix + R * B2 * PS + (SCMOS ? 2 * R : 0));
    stage_block<BOX, SCMOS>(a, spix, sok, R, roi0, nroi);

    const int g = threadIdx.x / TPR;  // ROI slot in the block
    const int r = threadIdx.x - g * TPR;
    const int rx = r % NCX, ry = r / NCX;
    const int c0 = (rx * BOX) / NCX, c1 = ((rx + 1) * BOX) / NCX;  // columns [c0, c1)
    const int r0 = (ry * BOX) / NRY;
    const int nr = ((ry + 1) * BOX) / NRY - r0;                     // rows [r0, r0 + nr)
    if (__all_sync(0xffffffffu, g >= nroi)) return;
    const bool valid = g < nroi && sok[g];
    const float *pix = spix + g * B2 * PS;
    // the lane's last row slot holds a row only when its block is a full RMAX
    const bool last_row = nr == RMAX;

    float th[P];
#pragma unroll
    for (int k = 0; k < P; k++) th[k] = 0.f;
    initialize<MODEL, BOX, PS>(pix, a.psf, th);
    // Poisson: the largest pixel of the ROI (NaN if any is NaN), for uncapped()
    float dmax = 0.f;
    if (!SCMOS) {
        dmax = -INFINITY;
        for (int j = c0; j < c1; j++)
            for (int t = 0; t < nr; t++) {
                const float d = pix[j * BOX + r0 + t];
                dmax = (d > dmax || d != d) ? d : dmax;
            }
#pragma unroll
        for (int off = TPR >> 1; off > 0; off >>= 1) {
            const float o = __shfl_xor_sync(0xffffffffu, dmax, off);
            dmax = (o > dmax || o != o) ? o : dmax;
        }
    }

    for (int it = 0; it <= a.iterations; ++it) {
        const bool final_pass = (it == a.iterations);
        float sxw, syw;
        AstigWidths aw;
        axis_widths<MODEL>(th, a, sxw, syw, aw);
        const float N = th[S::IN], bg = th[S::IB];
        const Axis ax = make_axis(th[S::IX], sxw, N, a.sqrt2pi, SIG);
        const Axis ay = make_axis(th[S::IY], syw, N, a.sqrt2pi, SIG);

        // this lane's rows of the y tables (slot t: row r0 + t + 1; a slot
        // past the block is evaluated but not used)
        float py[RMAX], yd1[RMAX], yd2[RMAX], ys1[SIG ? RMAX : 1], ys2[SIG ? RMAX : 1];
        {
            EdgeWalk wy = walk_start(r0 + 1, ay);
#pragma unroll
            for (int t = 0; t < RMAX; t++) {
                float s1 = 0.f, s2 = 0.f;
                walk_entry<SIG, true>(r0 + t + 1, ay, wy, py[t], yd1[t], yd2[t], s1, s2);
                if (SIG) { ys1[t] = s1; ys2[t] = s2; }
            }
        }
        EdgeWalk wx = walk_start(c0 + 1, ax);
        float xp, xd1, xd2, xs1 = 0.f, xs2 = 0.f;  // the lane's current column
        walk_entry<SIG, true>(c0 + 1, ax, wx, xp, xd1, xd2, xs1, xs2);

        if (!final_pass) {
            float py2[RMAX], aG[CROSS ? RMAX : 1], C[RMAX], D[RMAX];
#pragma unroll
            for (int t = 0; t < RMAX; t++) {
                py2[t] = py[t] * py[t];
                if (CROSS) aG[t] = py[t] * ys1[t];
                C[t] = 0.f;
                D[t] = 0.f;
            }
            float gs[P], hs[P];
#pragma unroll
            for (int k = 0; k < P; k++) { gs[k] = 0.f; hs[k] = 0.f; }
            auto columns = [&](auto uncapped_tag) {
                constexpr bool UNCAPPED = decltype(uncapped_tag)::value;
                for (int j = c0 + 1; j <= c1; j++) {
                    // next column's entry: independent of this column's pixels
                    float nxp, nxd1, nxd2, nxs1 = 0.f, nxs2 = 0.f;
                    walk_entry<SIG, true>(j + 1, ax, wx, nxp, nxd1, nxd2, nxs1, nxs2);
                    const float npx = N * xp, xp2 = xp * xp;
                    const float *col = pix + ((j - 1) * BOX + r0) * PS;
                    float A[2] = {0.f, 0.f}, B[2] = {0.f, 0.f}, E[2] = {0.f, 0.f},
                          F[2] = {0.f, 0.f}, Gc[2] = {0.f, 0.f};
#pragma unroll
                    for (int t = 0; t < RMAX; t++) {
                        if (t == RMAX - 1 && !last_row) break;
                        float d, v = 0.f;
                        if (SCMOS) {
                            const float2 q = reinterpret_cast<const float2 *>(col)[t];
                            d = q.x; v = q.y;
                        } else {
                            d = col[t];
                        }
                        const float mu = fmaf(npx, py[t], bg);
                        float cf, df;
                        if constexpr (UNCAPPED) likelihood_terms_uncapped(d, mu, cf, df);
                        else likelihood_terms<SCMOS>(d, v, mu, cf, df);
                        const int h = t & 1;
                        A[h] = fmaf(py[t], cf, A[h]);
                        B[h] = fmaf(py2[t], df, B[h]);
                        E[h] += cf;
                        F[h] += df;
                        C[t] = fmaf(xp, cf, C[t]);
                        D[t] = fmaf(xp2, df, D[t]);
                        if (CROSS) Gc[h] = fmaf(aG[t], df, Gc[h]);
                    }
                    col_terms<MODEL, P>(gs, hs, xp, xd1, xd2, xs1, xs2, A[0] + A[1],
                                        B[0] + B[1], E[0] + E[1], F[0] + F[1], Gc[0] + Gc[1],
                                        ax, aw);
                    xp = nxp; xd1 = nxd1; xd2 = nxd2; xs1 = nxs1; xs2 = nxs2;
                }
            };
            if constexpr (!SCMOS) {
                if (__all_sync(0xffffffffu, g >= nroi || uncapped(N, bg, dmax)))
                    columns(std::true_type{});
                else
                    columns(std::false_type{});
            } else {
                columns(std::false_type{});
            }
#pragma unroll
            for (int t = 0; t < RMAX; t++) {
                if (t == RMAX - 1 && !last_row) break;
                row_terms<MODEL, P>(gs, hs, yd1[t], yd2[t], SIG ? ys1[t] : 0.f,
                                    SIG ? ys2[t] : 0.f, C[t], D[t], ay, aw);
            }
#pragma unroll
            for (int k = 0; k < P; k++) {
                gs[k] = group_sum(gs[k], TPR);
                hs[k] = group_sum(hs[k], TPR);
            }
            newton_step<P>(th, gs, hs, a);
        } else {
            float llr = 0.f;
            float Fh[P][P], Fl[P][P];
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = 0; l < P; l++) { Fh[k][l] = 0.f; Fl[k][l] = 0.f; }
            for (int j = c0 + 1; j <= c1; j++) {
                float nxp, nxd1, nxd2, nxs1 = 0.f, nxs2 = 0.f;
                walk_entry<SIG, false>(j + 1, ax, wx, nxp, nxd1, nxd2, nxs1, nxs2);
                const float npx = N * xp;
                const float *col = pix + ((j - 1) * BOX + r0) * PS;
                float Q[NB][NB];
#pragma unroll
                for (int p = 0; p < NB; p++)
#pragma unroll
                    for (int q = 0; q < NB; q++) Q[p][q] = 0.f;
#pragma unroll
                for (int t = 0; t < RMAX; t++) {
                    if (t == RMAX - 1 && !last_row) break;
                    float d, v = 0.f;
                    if (SCMOS) {
                        const float2 q = reinterpret_cast<const float2 *>(col)[t];
                        d = q.x; v = q.y;
                    } else {
                        d = col[t];
                    }
                    const float mu = fmaf(npx, py[t], bg);
                    final_pixel<SCMOS, SIG, NB>(d, v, mu, py[t], yd1[t], SIG ? ys1[t] : 0.f,
                                                llr, Q);
                }
                fisher_column<MODEL, P, NB>(Fh, Fl, Q, xp, xd1, xs1, aw);
                xp = nxp; xd1 = nxd1; xs1 = nxs1;
            }
            llr = group_sum(llr, TPR);
            double Fm[P][P];
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = k; l < P; l++) {
                    dd_group_sum(Fh[k][l], Fl[k][l], TPR);
                    Fm[k][l] = dd_to_double(Fh[k][l], Fl[k][l]);
                    Fm[l][k] = Fm[k][l];
                }
            if (r == 0 && g < nroi) write_result<P>(a, roi0 + g, valid, th, Fm, llr);
        }
    }
}

// TABLE as for fit_kernel_r1; the launch's lanes per ROI are TPR (a.tpr).
template <int MODEL, int BOX, bool SCMOS, bool TABLE, int TPR>
__global__ void __launch_bounds__(256) fit_kernel(const KernelArgs a, const TileTable t)
{
    extern __shared__ __align__(16) float smem[];
    const int R = blockDim.x / TPR;
    if (!TABLE) {
        const int64_t roi0 = (int64_t)blockIdx.x * R;
        const int64_t left = a.n - roi0;
        fit_rois_tpr<MODEL, BOX, SCMOS, TPR>(a, roi0, left < R ? (int)left : R, smem);
        return;
    }
    TableSlot *ts = table_slot(smem, smem_bytes(MODEL, BOX, SCMOS, TPR, R));
    table_slot_init(ts);
    int64_t roi0;
    int nroi;
    for (int k = 0; table_next(t, R, ts, k, roi0, nroi); k++) {
        fit_rois_tpr<MODEL, BOX, SCMOS, TPR>(ts->a, roi0, nroi, smem);
        __syncthreads();  // the tile's shared memory and slot are free again
    }
}

}  // namespace gmle
