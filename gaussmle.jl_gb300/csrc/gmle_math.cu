// gmle_math.cu - the fit kernels' own elementary functions, evaluated for
// a check of their accuracy (gmle_math_selftest).
//
// The fit evaluates erf and exp at every pixel edge of every iteration, a
// reciprocal at every pixel and, in the Poisson final pass, two logarithms per
// pixel (gmle_fit_kernel.cuh: erf_from_gauss, gauss_edge, rcp_approx,
// log_approx).  This entry point evaluates them on caller-supplied arguments
// next to the CUDA library's erff, expf, IEEE division and logf, in the same
// kernel, so that a test can bound their error against those and against an
// FP64 reference on the host.
#include <cuda_runtime.h>

#include "gmle_fit_kernel.cuh"
#include "../../include/gaussmle_gb300.h"

namespace {

__global__ void math_selftest_kernel(const float *__restrict__ x, int64_t n, float *__restrict__ out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = x[i];
    // the fit's erf takes exp(-v^2) from gauss_edge at the same edge, whose
    // argument is the edge offset over sigma (here sqrt(2) v)
    const float e = gmle::gauss_edge(v * 1.41421356237309515f);
    out[i] = gmle::erf_from_gauss(v, e);
    out[n + i] = erff(v);
    out[2 * n + i] = gmle::gauss_edge(v);
    out[3 * n + i] = expf(-0.5f * (v * v));
    out[4 * n + i] = gmle::rcp_approx(v);
    out[5 * n + i] = __fdiv_rn(1.0f, v);
    // the Poisson LLR's logarithm at |x| (its arguments are positive)
    out[6 * n + i] = gmle::log_approx(fabsf(v));
    out[7 * n + i] = logf(fabsf(v));
}

}  // namespace

extern "C" gmle_status gmle_math_selftest(const float *d_x, int64_t n, float *d_out, void *stream)
{
    if (n < 0 || (n > 0 && (!d_x || !d_out))) return GMLE_INVALID_ARG;
    if (n == 0) return GMLE_OK;
    const int threads = 256;
    const int64_t blocks = (n + threads - 1) / threads;
    if (blocks > 0x7fffffffLL) return GMLE_INVALID_ARG;
    math_selftest_kernel<<<(unsigned)blocks, threads, 0, static_cast<cudaStream_t>(stream)>>>(
        d_x, n, d_out);
    return cudaGetLastError() == cudaSuccess ? GMLE_OK : GMLE_CUDA_ERROR;
}
