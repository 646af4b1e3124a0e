"""The fit kernels' own erf, exp and reciprocal against CUDA's and FP64.

The fit evaluates erf and exp once per pixel edge and a reciprocal once per
pixel (gmle_fit_kernel.cuh: erf_from_gauss, gauss_edge, rcp_approx) instead of
the library's erff (28 issued instructions), expf (9) and __fdividef (4), and
the Poisson final pass's two logarithms per pixel by log_approx instead of
logf (26).  Bounds checked here, on a dense grid and at the pixel-edge
arguments of the fits (|x| up to 8 pixel sigmas):
  * erf: within 5e-7 absolute of the FP64 erf (measured 4.3e-7, near x = 0;
    erff: 6e-8), within 6e-7 of erff;
  * exp(-x^2/2): within 4 ulp plus 6e-8 x^2 relative (the exponent's
    rounding) where above 1e-30;
  * 1/x: within 1 ulp of the IEEE quotient;
  * ln x (photon counts and model values, 1e-6 to 1e7, and subnormals):
    within 3e-7 absolute plus 2 ulp of the FP64 logarithm.
"""
import ctypes as C

import numpy as np
import pytest
from scipy.special import erf

pytestmark = pytest.mark.gpu


def run(ctx, x):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    xd = torch.from_numpy(np.ascontiguousarray(x, np.float32)).to(dev)
    out = torch.empty((8, len(x)), device=dev)
    ctx.check(ctx.lib.gmle_math_selftest(C.c_void_p(xd.data_ptr()), len(x),
                                         C.c_void_p(out.data_ptr()), None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_erf_exp_rcp_accuracy(ctx):
    x = np.concatenate([np.linspace(-8, 8, 400_001),
                        np.random.default_rng(3).uniform(-6, 6, 200_000)]).astype(np.float32)
    o = run(ctx, x)
    ref = erf(x.astype(np.float64))
    e_fast = np.abs(o[0] - ref)
    e_lib = np.abs(o[1] - ref)
    print(f"\nerf: fit max |err| {e_fast.max():.3e}, erff max |err| {e_lib.max():.3e}")
    assert e_fast.max() <= 5e-7
    assert np.abs(o[0] - o[1]).max() <= 6e-7
    # the sign is right except within the error bound of 0 (erf(x) ~ 1.13 x
    # for |x| < 1e-7, where 1 - e t P(t) rounds to +-6e-8)
    wrong = np.sign(o[0]) != np.sign(x)
    assert np.all(np.abs(o[0][wrong]) <= 1.2e-7) and np.all(np.abs(x[wrong]) <= 1e-6)
    g = np.exp(-0.5 * x.astype(np.float64) ** 2)
    big = g > 1e-30
    rel = np.abs(o[2][big] - g[big]) / g[big]
    print(f"exp(-x^2/2): fit max rel {rel.max():.3e}, expf max rel "
          f"{(np.abs(o[3][big] - g[big]) / g[big]).max():.3e}")
    # 4 ulp, plus the rounding of the exponent x^2 log2(e) / 2 (half an ulp of
    # it, relative error ln 2 times that): 6e-8 x^2, which only the far tail
    # reaches (x = 8: value 1e-14, error 2.6e-6 relative)
    xb = x[big].astype(np.float64)
    assert np.all(rel <= 2.5e-7 + 6e-8 * xb * xb)
    nz = x != 0
    ulp = np.spacing(np.abs(o[5][nz]).astype(np.float32))
    assert np.all(np.abs(o[4][nz] - o[5][nz]) <= ulp)


def test_erf_is_monotone_and_odd(ctx):
    x = np.linspace(0, 6, 1_000_001).astype(np.float32)
    o = run(ctx, np.concatenate([x, -x]))
    pos, neg = o[0][: len(x)], o[0][len(x):]
    assert np.array_equal(pos, -neg)
    # increasing up to rounding: no step back larger than 2 ulp of 1
    assert np.diff(pos).min() >= -2.5e-7


def test_log_accuracy(ctx):
    rng = np.random.default_rng(5)
    x = np.concatenate([np.geomspace(1e-6, 1e7, 400_001), rng.uniform(0.5, 2e4, 200_000),
                        np.arange(1, 20_001), [1e-40, 1e-44, 3e38]]).astype(np.float32)
    o = run(ctx, x)
    ref = np.log(x.astype(np.float64))
    err = np.abs(o[6] - ref)
    lib = np.abs(o[7] - ref)
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    print(f"\nln: fit max |err| {err.max():.3e} (max in ulp {(err / ulp).max():.2f}), "
          f"logf max |err| {lib.max():.3e}")
    assert np.all(err <= 3e-7 + 2 * ulp)
