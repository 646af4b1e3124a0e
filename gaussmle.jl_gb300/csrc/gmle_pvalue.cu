// gmle_pvalue.cu - goodness-of-fit p-values of the fits, on the device.
//
// The reference computes them on the host after every fit, one ROI at a time
// (src/interface.jl:265-275, :459-468):
//     chi2 = -2 llr            (Float32)
//     p    = 1 - Float32(cdf(Chisq(df), chi2)),   df = box^2 - P.
// cdf(Chisq(df), x) is the regularised lower incomplete gamma function
// P(df/2, x/2), evaluated by Distributions.jl in Float64 (the Float32 chi2 is
// promoted and halved exactly).  Here P(a, x) is evaluated in FP64 by the
// classical scheme (Numerical Recipes, 2nd ed., sec. 6.2; Abramowitz & Stegun
// 6.5.29 and 6.5.31): the power series
//     P = x^a e^-x / Gamma(a) * sum_n x^n / (a (a+1) ... (a+n))      (x < a + 1)
// and otherwise the continued fraction of Q = 1 - P, evaluated with the
// modified Lentz method.  Both loops stop at a relative term below 1e-16 or
// after 1000 terms; the p-value is then rounded to Float32 as the reference
// does.  One thread per ROI; the cost (a few hundred FP64 operations per ROI)
// is small next to the fit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "gmle_internal.h"

namespace {

__device__ double gamma_p(double a, double x)
{
    if (isnan(x)) return x;
    if (x <= 0.0) return 0.0;  // Distributions clamps x at 0: P(a, 0) = 0
    if (isinf(x)) return 1.0;
    const double log_pre = a * log(x) - x - lgamma(a);  // log(x^a e^-x / Gamma(a))
    if (x < a + 1.0) {
        double ap = a, term = 1.0 / a, sum = term;
        for (int n = 0; n < 1000; n++) {
            ap += 1.0;
            term *= x / ap;
            sum += term;
            if (fabs(term) < fabs(sum) * 1e-16) break;
        }
        return sum * exp(log_pre);
    }
    const double tiny = 1e-300;
    double b = x + 1.0 - a, c = 1.0 / tiny, d = 1.0 / b, h = d;
    for (int i = 1; i < 1000; i++) {
        const double an = -i * (i - a);
        b += 2.0;
        d = an * d + b;
        if (fabs(d) < tiny) d = tiny;
        c = b + an / c;
        if (fabs(c) < tiny) c = tiny;
        d = 1.0 / d;
        const double del = d * c;
        h *= del;
        if (fabs(del - 1.0) < 1e-16) break;
    }
    return 1.0 - exp(log_pre) * h;
}

__global__ void pvalue_kernel(const float *__restrict__ llr, int64_t n, double a,
                              float *__restrict__ pvalues)
{
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const float chi2 = -2.0f * llr[k];
        pvalues[k] = 1.0f - (float)gamma_p(a, 0.5 * (double)chi2);
    }
}

gmle_status launch_pvalues(gmle_ctx *ctx, const float *d_llr, int64_t n, int32_t df,
                           float *d_pvalues, cudaStream_t s)
{
    if (n <= 0) return GMLE_OK;
    const int threads = 256;
    const int64_t blocks = std::min<int64_t>((n + threads - 1) / threads,
                                             (int64_t)ctx->num_sms * 8);
    ctx->launches++;
    pvalue_kernel<<<(unsigned)blocks, threads, 0, s>>>(d_llr, n, 0.5 * (double)df, d_pvalues);
    GMLE_CK(cudaGetLastError(), "p-value kernel launch");
    return GMLE_OK;
}

gmle_status check_pvalue_args(gmle_ctx *ctx, const float *llr, int64_t n, int32_t df,
                              const float *pvalues)
{
    if (n < 0) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "n < 0");
    if (n > 0 && (!llr || !pvalues))
        return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "llr and pvalues are required");
    if (df <= 0) return gmle_rt::fail(ctx, GMLE_INVALID_ARG, "degrees of freedom must be > 0");
    return GMLE_OK;
}

}  // namespace

extern "C" gmle_status gmle_pvalues_device(gmle_ctx *ctx, const float *d_llr, int64_t n,
                                           int32_t df, float *d_pvalues, void *stream)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    gmle_status st = check_pvalue_args(ctx, d_llr, n, df, d_pvalues);
    if (st != GMLE_OK) return st;
    cudaSetDevice(ctx->device);
    return launch_pvalues(ctx, d_llr, n, df, d_pvalues, static_cast<cudaStream_t>(stream));
}

extern "C" gmle_status gmle_pvalues(gmle_ctx *ctx, const float *llr, int64_t n, int32_t df,
                                    float *pvalues)
{
    if (!ctx) return GMLE_INVALID_ARG;
    std::lock_guard<std::mutex> lk(ctx->mu);
    gmle_status st = check_pvalue_args(ctx, llr, n, df, pvalues);
    if (st != GMLE_OK || n == 0) return st;
    cudaSetDevice(ctx->device);
    if (ctx->pv_cap < n) {
        cudaFree(ctx->d_pv);
        ctx->d_pv = nullptr;
        ctx->pv_cap = 0;
        GMLE_CK(cudaMalloc(&ctx->d_pv, 2 * sizeof(float) * (size_t)n), "cudaMalloc(p-values)");
        ctx->pv_cap = n;
    }
    float *d_in = ctx->d_pv, *d_out = ctx->d_pv + n;
    cudaStream_t s = ctx->s_fit;
    GMLE_CK(cudaMemcpyAsync(d_in, llr, sizeof(float) * (size_t)n, cudaMemcpyHostToDevice, s),
            "H2D llr");
    st = launch_pvalues(ctx, d_in, n, df, d_out, s);
    if (st != GMLE_OK) return st;
    GMLE_CK(cudaMemcpyAsync(pvalues, d_out, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, s),
            "D2H p-values");
    GMLE_CK(cudaStreamSynchronize(s), "cudaStreamSynchronize");
    return GMLE_OK;
}
