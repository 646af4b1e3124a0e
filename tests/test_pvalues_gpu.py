"""Goodness-of-fit p-values on the GPU (gmle_pvalues, gmle_pvalues_device)
against the reference's formula (src/interface.jl:265-275) in the oracle."""
import ctypes as C

import numpy as np
import pytest

import gaussmle_gb300 as G
from oracle import oracle as O
from parity_cases import make_case

pytestmark = pytest.mark.gpu

# Float32 rounding of a cdf that is correct to ~1e-15: at most one ulp of 1.
TOL = 1.2e-7


def _gpu(ctx, llr, df):
    llr = np.ascontiguousarray(llr, np.float32)
    out = np.full_like(llr, -1.0)
    ctx.check(ctx.lib.gmle_pvalues(ctx.handle, llr.ctypes.data_as(C.c_void_p), llr.size, df,
                                   out.ctypes.data_as(C.c_void_p)))
    return out


@pytest.mark.parametrize("df", [1, 2, 7, 45, 117, 164, 220])
def test_pvalues_match_the_reference_formula(ctx, df):
    rng = np.random.default_rng(df)
    # chi2 around and far from its mean df (both branches of the evaluation)
    chi2 = np.concatenate([rng.chisquare(df, 20000), rng.uniform(0, 6 * df + 50, 5000),
                           [0.0, 1e-30, 0.5 * df, df + 2.0, 1e4]]).astype(np.float32)
    llr = (-0.5 * chi2).astype(np.float32)
    np.testing.assert_allclose(_gpu(ctx, llr, df), O.pvalues(llr, df), rtol=0, atol=TOL)


def test_pvalue_edge_values(ctx):
    llr = np.array([0.0, 5.0, np.nan, -np.inf, -1e6], np.float32)
    got = _gpu(ctx, llr, 117)
    assert got[0] == 1.0 and got[1] == 1.0  # chi2 <= 0
    assert np.isnan(got[2])
    assert got[3] == 0.0 and got[4] == 0.0
    assert ctx.lib.gmle_pvalues(ctx.handle, None, 3, 117, None) == 1
    assert ctx.lib.gmle_pvalues(ctx.handle, llr.ctypes.data_as(C.c_void_p), 5, 0,
                                llr.ctypes.data_as(C.c_void_p)) == 1


def test_fit_pvalues_come_from_the_device_and_match_the_oracle(ctx):
    w = make_case("xynb-11-poisson", 0, 11, 0, 3000)
    fitter = G.GaussMLEFitter(psf_model=G.GaussianXYNB(0.13))
    l0 = fitter.context.launches()
    res = G.fit(fitter, w.data)
    assert fitter.context.launches() - l0 >= 2  # the fit and the p-value kernel
    np.testing.assert_allclose(res.pvalues, O.pvalues(res.log_likelihoods, 121 - 4), rtol=0,
                               atol=TOL)
    # well-specified Poisson fits: p-values spread over (0, 1)
    assert 0.2 < float(np.median(res.pvalues)) < 0.8


def test_device_entry_on_a_stream(ctx):
    torch = pytest.importorskip("torch")
    llr = np.linspace(-300, 0, 4097, dtype=np.float32)
    d_llr = torch.from_numpy(llr).cuda()
    d_pv = torch.empty_like(d_llr)
    s = torch.cuda.Stream()
    ctx.check(ctx.lib.gmle_pvalues_device(ctx.handle, C.c_void_p(d_llr.data_ptr()), llr.size, 45,
                                          C.c_void_p(d_pv.data_ptr()), C.c_void_p(s.cuda_stream)))
    s.synchronize()
    np.testing.assert_allclose(d_pv.cpu().numpy(), O.pvalues(llr, 45), rtol=0, atol=TOL)
