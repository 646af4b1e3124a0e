"""CPU checks of the oracle (the checker of the CUDA path).

* Its CRLB code agrees with the reference's own first-principles Fisher /
  CRLB derivation (dev/astig_theory/compute_theoretical_crlb.jl, restated in
  tests/golden/make_golden.py).
* It reproduces its committed golden fixtures.
* It passes the reference test-suite's statistical acceptance protocols
  (tests/statistics_cases.py).
* FP32 and FP64 builds agree for well-conditioned fits.
"""
from pathlib import Path

import numpy as np
import pytest

import statistics_cases as SC
from oracle import oracle as O

GOLDEN = Path(__file__).resolve().parent / "golden"


def oracle_fit(model, box, camera, psf, data, xc, yc, maps, cons, precision="f32"):
    d = O.make_desc(model, box, 20, camera, psf.psf_vector(), cons.lower, cons.upper,
                    cons.max_step)
    r = O.fit(d, data, xc, yc, maps, precision)
    return r["params"], r["crlb"]


@pytest.mark.parametrize("precision,rtol", [("f64", 1e-6), ("f32", 2e-3)])
def test_crlb_matches_reference_theory_derivation(precision, rtol):
    g = np.load(GOLDEN / "astig_theory_crlb.npz")
    for th, ref in zip(g["theta"], g["crlb"]):
        got, flags = O.crlb_at(3, int(g["box"]), g["psf"], th, precision)
        assert flags & O.FLAG_CONVERGED
        np.testing.assert_allclose(got, ref, rtol=rtol)


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("oracle_*.npz")), ids=lambda p: p.stem)
def test_oracle_reproduces_golden_fixture(path):
    g = np.load(path)
    maps = (g["var"], g["gain"], g["offset"]) if int(g["camera"]) else None
    d = O.make_desc(int(g["model"]), int(g["box"]), 20, int(g["camera"]), g["psf"], g["lower"],
                    g["upper"], g["max_step"])
    r = O.fit(d, g["data"], g["xc"], g["yc"], maps, "f32")
    np.testing.assert_allclose(r["params"], g["params"], rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(r["crlb"], g["crlb"], rtol=1e-5)
    np.testing.assert_allclose(r["llr"], g["llr"], rtol=1e-5, atol=1e-5)
    assert np.array_equal(r["flags"], g["flags"])


@pytest.mark.parametrize("model", [0, 1, 2], ids=["xynb", "xynbs", "xynbsxsy"])
def test_model_validation_protocol(model):
    res = SC.check_model_validation(oracle_fit, model)
    assert all(v["pass"] for v in res.values()), res


def test_astigmatic_validation_protocol():
    """test/model_validation_tests.jl:97-135 on the FP32 oracle."""
    res = SC.check_astig_validation(oracle_fit)
    assert all(v["pass"] for v in res.values()), res


def test_scmos_photometry_protocol():
    res = SC.check_scmos_photometry(oracle_fit)
    assert res["pass"], res


def test_scmos_variance_map_indexing_protocol():
    res = SC.check_variance_indexing(oracle_fit)
    assert res["pass"], res


def test_precision_improves_with_photons():
    res = SC.check_precision_vs_photons(oracle_fit)
    assert res["pass"], res


def test_fp32_and_fp64_builds_agree_when_well_conditioned():
    psf, truth, data = SC.model_validation_data(0, n=300, box=11, seed=9)
    from gaussmle_gb300.constraints import default_constraints
    cons = default_constraints(psf, 11)
    ones = np.ones(300, np.int32)
    p32, c32 = oracle_fit(0, 11, 0, psf, data, ones, ones, None, cons, "f32")
    p64, c64 = oracle_fit(0, 11, 0, psf, data, ones, ones, None, cons, "f64")
    assert np.abs(p32[:, :2] - p64[:, :2]).max() < 1e-4
    np.testing.assert_allclose(c32, c64, rtol=1e-4)


def test_oracle_rejects_bad_descriptors():
    d = O.make_desc(7, 11, 20, 0, np.zeros(8), [0] * 4, [1] * 4, [1] * 4)
    with pytest.raises(ValueError):
        O.fit(d, np.zeros((11, 11, 1), np.float32))
    d = O.make_desc(0, 2, 20, 0, np.zeros(8), [0] * 4, [1] * 4, [1] * 4)
    with pytest.raises(ValueError):
        O.fit(d, np.zeros((2, 2, 1), np.float32))


def test_zero_iterations_returns_the_initial_estimate():
    psf, truth, data = SC.model_validation_data(0, n=10, box=11, seed=3)
    from gaussmle_gb300.constraints import default_constraints
    c = default_constraints(psf, 11)
    d = O.make_desc(0, 11, 0, 0, psf.psf_vector(), c.lower, c.upper, c.max_step)
    r = O.fit(d, data)
    # the reference initialisation (src/unified_kernel.jl:158-192): bg = mean of
    # the edge pixels, photons = max(sum(max(0, d - bg)), 100)
    roi = np.asarray(data[:, :, 0], np.float64)
    edge = np.concatenate([roi[0, :], roi[-1, :], roi[1:-1, 0], roi[1:-1, -1]])
    assert abs(r["params"][0, 3] - edge.mean()) < 1e-3
    sig = np.maximum(0, roi - edge.mean()).sum()
    assert abs(r["params"][0, 2] - max(sig, 100)) / max(sig, 100) < 1e-5


def test_oracle_pvalues_known_answers():
    """The p-value formula of src/interface.jl:265-275 on closed forms and the
    5% critical values of the chi-square distribution."""
    x = np.array([0.0, 1.0, 4.0, 10.0])
    llr = (-0.5 * x).astype(np.float32)
    # df = 2: cdf(x) = 1 - exp(-x/2), so p = 1 - Float32(1 - exp(-x/2))
    want = np.float32(1) - (1 - np.exp(-0.5 * x)).astype(np.float32)
    np.testing.assert_array_equal(O.pvalues(llr, 2), want)
    for df, crit in ((1, 3.841459), (10, 18.307038)):
        p = O.pvalues(np.array([-0.5 * crit], np.float32), df)[0]
        assert abs(p - 0.05) < 2e-6, (df, p)
    assert np.isnan(O.pvalues(np.array([np.nan], np.float32), 5)[0])
    assert O.pvalues(np.array([3.0], np.float32), 5)[0] == 1.0  # chi2 < 0 clamps to 0


def _lm_vs_newton(name, model, box, camera, n):
    import sys
    from parity_cases import make_case, oracle_desc
    w = make_case(name, model, box, camera, n)
    dn = oracle_desc(O, w)
    dl = oracle_desc(O, w)
    dl.method = 1
    rn = O.fit(dn, w.data, w.x_corners, w.y_corners, w.maps, "f32")
    rl = O.fit(dl, w.data, w.x_corners, w.y_corners, w.maps, "f32")
    return rn, rl


def test_full_hessian_option_equals_newton_when_well_posed():
    """The full-Hessian option (Fisher scoring with LM damping, an extension)
    reaches the same maximum as the reference's Newton step on well-posed
    XYNB fits: positions within 1e-3 px, the same flags."""
    rn, rl = _lm_vs_newton("xynb-11-poisson", 0, 11, 0, 300)
    assert np.array_equal(rn["flags"], rl["flags"])
    assert np.abs(rn["params"][:, :2] - rl["params"][:, :2]).max() < 1e-3


@pytest.mark.parametrize("case", [("xynbs-13-scmos-adu", 1, 13, 2, 200),
                                  ("xynbsxsy-13-scmos-adu", 2, 13, 2, 200)])
def test_full_hessian_option_reaches_higher_likelihood_on_sigma_models(case):
    """With the sigma models 20 reference Newton steps stop short of the
    maximum; the full-Hessian option's log-likelihood is at least theirs."""
    rn, rl = _lm_vs_newton(*case)
    d = rl["llr"] - rn["llr"]
    assert np.mean(d >= -1e-2) > 0.97 and d.mean() > 0
