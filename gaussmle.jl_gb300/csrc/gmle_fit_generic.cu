// gmle_fit_generic.cu - the fit for ROIs larger than the specialised kernels
// take (box 17..64): the same iteration as fit_kernel_r1
// (src/unified_kernel.jl:285-434) with the box a run-time value.
//
// The reference fits any square ROI of at least 3 pixels (src/interface.jl:22;
// its kernel is generic in the box, src/unified_kernel.jl:300).  Boxes 3..16
// run in the specialised kernels (gmle_launch.cuh); this kernel covers the
// rest up to 64, at a lower rate: one thread per ROI, and the ROI's pixels,
// its variance tile and its axis tables and row sums in shared memory, element
// e of slot g at [e * R + g] (conflict-free: consecutive threads, consecutive
// words), with loops over the run-time box.
#include <cuda_runtime.h>

#include "gmle_fit_kernel.cuh"
#include "gmle_generic.h"

namespace gmle {

namespace {

// floats of shared memory per ROI slot
__host__ __device__ inline int generic_floats(int box, bool scmos)
{
    return box * box * (scmos ? 2 : 1) + 7 * box;
}

template <int MODEL, bool SCMOS>
__global__ void __launch_bounds__(128) fit_kernel_generic(const KernelArgs a, const int box)
{
    constexpr int P = ModelInfo<MODEL>::P;
    constexpr bool SIG = ModelInfo<MODEL>::SIG;
    constexpr bool CROSS = (MODEL == 1 || MODEL == 3);
    constexpr int NB = SIG ? 4 : 3;
    using S = Slots<MODEL>;
    extern __shared__ __align__(16) float smem[];
    const int R = blockDim.x, g = threadIdx.x;
    const int B2 = box * box;
    const int64_t roi0 = (int64_t)blockIdx.x * R;
    const int nroi = (int)min((int64_t)R, a.n - roi0);
    float *spix = smem;                                  // [B2][R]
    float *svar = spix + (size_t)B2 * R;                 // [B2][R], sCMOS
    float *stab = svar + (SCMOS ? (size_t)B2 * R : 0);   // [7 box][R]
    auto PIX = [&](int p) -> float & { return spix[(size_t)p * R + g]; };
    auto VAR = [&](int p) -> float & { return svar[(size_t)p * R + g]; };
    // tables: 0 psf_y, 1 d psf_y, 2 d2 psf_y, 3 ds psf_y, 4 d2s psf_y, 5 C, 6 D
    auto TAB = [&](int k, int t) -> float & { return stab[((size_t)k * box + t) * R + g]; };

    // pixels: the block's ROIs are contiguous in global memory
    const float *src = a.data + roi0 * B2;
    for (int e = threadIdx.x; e < nroi * B2; e += R) {
        const int q = e / B2, p = e - q * B2;
        spix[(size_t)p * R + q] = src[e];
    }
    __syncthreads();
    if (g >= nroi) return;  // no barrier follows
    bool valid = true;
    if (SCMOS) {
        const int32_t x0 = a.xc[roi0 + g], y0 = a.yc[roi0 + g];
        valid = x0 >= 1 && y0 >= 1 && x0 + box - 1 <= a.nx && y0 + box - 1 <= a.ny;
        if (!valid) atomicAdd(a.bad_corners, 1ull);
        const long long base = valid ? (long long)(y0 - 1) + (long long)a.ny * (x0 - 1) : 0;
        for (int j = 0; j < box; j++)
            for (int i = 0; i < box; i++) {
                const int p = i + box * j;
                const long long m = base + i + (long long)a.ny * j;
                VAR(p) = valid ? __ldg(a.var + m) : 0.f;
                // (ADU - offset) * gain, src/camera_models.jl:110-113
                if (valid && a.adu) PIX(p) = __fmul_rn(__fadd_rn(PIX(p), -__ldg(a.offset + m)),
                                                       __ldg(a.gain + m));
            }
    }

    float th[P];
#pragma unroll
    for (int k = 0; k < P; k++) th[k] = 0.f;
    initialize_box<MODEL>(box, [&](int p) { return PIX(p); }, a.psf, th);

    for (int it = 0; it <= a.iterations; ++it) {
        const bool final_pass = (it == a.iterations);
        float sxw, syw;
        AstigWidths aw;
        axis_widths<MODEL>(th, a, sxw, syw, aw);
        const float N = th[S::IN], bg = th[S::IB];
        const Axis ax = make_axis(th[S::IX], sxw, N, a.sqrt2pi, SIG);
        const Axis ay = make_axis(th[S::IY], syw, N, a.sqrt2pi, SIG);
        {
            EdgeWalk wy = walk_start(1, ay);
            for (int t = 0; t < box; t++) {
                float p, d1, d2, s1 = 0.f, s2 = 0.f;
                walk_entry<SIG, true>(t + 1, ay, wy, p, d1, d2, s1, s2);
                TAB(0, t) = p;
                TAB(1, t) = d1;
                TAB(2, t) = d2;
                TAB(3, t) = s1;
                TAB(4, t) = s2;
                TAB(5, t) = 0.f;
                TAB(6, t) = 0.f;
            }
        }
        EdgeWalk wx = walk_start(1, ax);
        if (!final_pass) {
            float gs[P], hs[P];
#pragma unroll
            for (int k = 0; k < P; k++) { gs[k] = 0.f; hs[k] = 0.f; }
            for (int j = 1; j <= box; j++) {
                float xp, xd1, xd2, xs1 = 0.f, xs2 = 0.f;
                walk_entry<SIG, true>(j, ax, wx, xp, xd1, xd2, xs1, xs2);
                const float npx = N * xp, xp2 = xp * xp;
                float A = 0.f, B = 0.f, E = 0.f, F = 0.f, Gc = 0.f;
                for (int t = 0; t < box; t++) {
                    const int p = t + box * (j - 1);
                    const float py = TAB(0, t);
                    const float mu = fmaf(npx, py, bg);
                    float cf, df;
                    likelihood_terms<SCMOS>(PIX(p), SCMOS ? VAR(p) : 0.f, mu, cf, df);
                    A = fmaf(py, cf, A);
                    B = fmaf(py * py, df, B);
                    E += cf;
                    F += df;
                    TAB(5, t) = fmaf(xp, cf, TAB(5, t));
                    TAB(6, t) = fmaf(xp2, df, TAB(6, t));
                    if (CROSS) Gc = fmaf(py * TAB(3, t), df, Gc);
                }
                col_terms<MODEL, P>(gs, hs, xp, xd1, xd2, xs1, xs2, A, B, E, F, Gc, ax, aw);
            }
            for (int t = 0; t < box; t++)
                row_terms<MODEL, P>(gs, hs, TAB(1, t), TAB(2, t), TAB(3, t), TAB(4, t), TAB(5, t),
                                    TAB(6, t), ay, aw);
            newton_step<P>(th, gs, hs, a);
        } else {
            float llr = 0.f;
            float Fh[P][P], Fl[P][P];
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = 0; l < P; l++) { Fh[k][l] = 0.f; Fl[k][l] = 0.f; }
            for (int j = 1; j <= box; j++) {
                float xp, xd1, xd2, xs1 = 0.f, xs2 = 0.f;
                walk_entry<SIG, false>(j, ax, wx, xp, xd1, xd2, xs1, xs2);
                const float npx = N * xp;
                float Q[NB][NB];
#pragma unroll
                for (int q = 0; q < NB; q++)
#pragma unroll
                    for (int r = 0; r < NB; r++) Q[q][r] = 0.f;
                for (int t = 0; t < box; t++) {
                    const int p = t + box * (j - 1);
                    const float py = TAB(0, t);
                    const float mu = fmaf(npx, py, bg);
                    final_pixel<SCMOS, SIG, NB>(PIX(p), SCMOS ? VAR(p) : 0.f, mu, py, TAB(1, t),
                                                TAB(3, t), llr, Q);
                }
                fisher_column<MODEL, P, NB>(Fh, Fl, Q, xp, xd1, xs1, aw);
            }
            double Fm[P][P];
#pragma unroll
            for (int k = 0; k < P; k++)
#pragma unroll
                for (int l = k; l < P; l++) {
                    Fm[k][l] = dd_to_double(Fh[k][l], Fl[k][l]);
                    Fm[l][k] = Fm[k][l];
                }
            write_result<P>(a, roi0 + g, valid, th, Fm, llr);
        }
    }
}

using GenericKernel = void (*)(const KernelArgs, const int);

GenericKernel generic_kernel(int model, bool scmos)
{
    switch (model * 2 + (int)scmos) {
        case 0: return fit_kernel_generic<0, false>;
        case 1: return fit_kernel_generic<0, true>;
        case 2: return fit_kernel_generic<1, false>;
        case 3: return fit_kernel_generic<1, true>;
        case 4: return fit_kernel_generic<2, false>;
        case 5: return fit_kernel_generic<2, true>;
        case 6: return fit_kernel_generic<3, false>;
        case 7: return fit_kernel_generic<3, true>;
        default: return nullptr;
    }
}

}  // namespace

int generic_rois_per_block(int box, bool scmos)
{
    const size_t per_roi = sizeof(float) * (size_t)generic_floats(box, scmos);
    int r = 128;
    while (r > 1 && per_roi * r > 200 * 1024) r /= 2;
    return r;
}

cudaError_t launch_fit_generic(int model, int box, bool scmos, const KernelArgs &a, cudaStream_t s)
{
    if (box < kGenericMinBox || box > kGenericMaxBox) return cudaErrorInvalidValue;
    GenericKernel k = generic_kernel(model, scmos);
    if (!k) return cudaErrorInvalidValue;
    const int rpb = generic_rois_per_block(box, scmos);
    const size_t smem = sizeof(float) * (size_t)generic_floats(box, scmos) * rpb;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         227 * 1024);
    if (e != cudaSuccess) return e;
    const int64_t blocks = (a.n + rpb - 1) / rpb;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    k<<<(unsigned)blocks, rpb, smem, s>>>(a, box);
    return cudaGetLastError();
}

}  // namespace gmle
