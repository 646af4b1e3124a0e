"""The device ROI generator (gmle_simulate_device) against its CPU restatement
(oracle/simulate_oracle.py), the Poisson and sCMOS noise laws, and the fit on
data the generator makes, to the reference's own validation bars: std/CRLB
within 10% for Poisson data (test/validation_utils.jl:341-350,
test/model_validation_tests.jl:6-135) and within 30% for sCMOS data, whose
Newton step uses a Gaussian approximation (test/model_validation_tests.jl:
274-280)."""
import ctypes as C

import numpy as np
import pytest

import gaussmle_gb300 as G
from gaussmle_gb300.fitter import make_desc
from oracle import simulate_oracle as S
from parity_cases import make_case

pytestmark = pytest.mark.gpu

CASES = [("xynb-11", 0, 11), ("xynbs-9", 1, 9), ("xynbsxsy-13", 2, 13), ("astig-15", 3, 15),
         ("xynb-7", 0, 7)]


def _maps(ctx, maps):
    var, gain, off = (np.asfortranarray(m, np.float32) for m in maps)
    ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, var.ctypes.data_as(C.c_void_p),
                                           gain.ctypes.data_as(C.c_void_p),
                                           off.ctypes.data_as(C.c_void_p), var.shape[0],
                                           var.shape[1]))


def _gen(torch, ctx, w, camera, truth, seed, xc=None, yc=None):
    desc = make_desc(w.psf, w.box, 20, w.constraints, camera)
    t = torch.from_numpy(np.ascontiguousarray(truth, np.float32)).cuda()
    cx = torch.from_numpy(xc).cuda() if xc is not None else None
    cy = torch.from_numpy(yc).cuda() if yc is not None else None
    out = G.simulate_rois(ctx, desc, t, seed, cx, cy)
    torch.cuda.synchronize()
    n, b = truth.shape[0], w.box
    return out.cpu().numpy().reshape(n, b, b).transpose(2, 1, 0)  # (box, box, n), [i, j, k]


@pytest.mark.parametrize("camera", [0, 1, 2], ids=["poisson", "scmos-e", "scmos-adu"])
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_generator_matches_restatement(ctx, case, camera):
    """Draw for draw.  The float exp, log and cos of the device and of the host
    library may differ by an ulp, which moves a draw only when a uniform falls
    within that of a decision boundary: at most 1 in 10^4 Poisson counts may
    differ, and sCMOS values agree to float rounding."""
    torch = pytest.importorskip("torch")
    name, model, box = case
    w = make_case(name, model, box, 2, 24, seed=31 + model)
    truth = w.truth.copy()
    truth[:, 3 if model == 3 else 2] = np.geomspace(30, 20000, 24)  # both sampler branches
    _maps(ctx, w.maps)
    got = _gen(torch, ctx, w, camera, truth, 1234, w.x_corners, w.y_corners)
    ref = S.simulate(model, box, camera, np.asarray(w.psf.psf_vector(), np.float32), truth,
                     1234, tuple(np.asarray(m, np.float32) for m in w.maps), w.x_corners,
                     w.y_corners)
    if camera == 0:
        assert np.mean(got != ref) <= 1e-4
    else:
        close = np.isclose(got, ref, rtol=1e-5, atol=1e-4)
        assert np.mean(~close) <= 1e-4


def test_generator_is_deterministic_and_counter_based(ctx):
    torch = pytest.importorskip("torch")
    w = make_case("xynb-11", 0, 11, 0, 3000, seed=5)
    a = _gen(torch, ctx, w, 0, w.truth, 99)
    b = _gen(torch, ctx, w, 0, w.truth, 99)
    c = _gen(torch, ctx, w, 0, w.truth, 100)
    d = _gen(torch, ctx, w, 0, w.truth[:1700], 99)  # fewer ROIs: other blocks, same draws
    assert np.array_equal(a, b)
    assert np.mean(a != c) > 0.5
    assert np.array_equal(a[:, :, :1700], d)


@pytest.mark.parametrize("camera", [0, 1], ids=["poisson", "scmos-e"])
def test_pixel_moments(ctx, camera):
    """200 000 copies of one emitter: per-pixel mean mu and variance mu
    (+ the read-noise variance for sCMOS)."""
    torch = pytest.importorskip("torch")
    w = make_case("xynb-11", 0, 11, 2, 4, seed=8)
    _maps(ctx, w.maps)
    n = 200_000
    theta = np.array([6.2, 5.7, 3000.0, 12.0], np.float32)
    truth = np.tile(theta, (n, 1))
    xc = np.full(n, 40, np.int32)
    yc = np.full(n, 70, np.int32)
    got = _gen(torch, ctx, w, camera, truth, 7, xc, yc).astype(np.float64)
    mu = S.expectation64(0, np.asarray(w.psf.psf_vector(), np.float32), theta, 11)
    var = mu.copy()
    if camera:
        var += np.asarray(w.maps[0], np.float64)[69:80, 39:50]
    mean, v = got.mean(axis=2), got.var(axis=2)
    assert np.all(np.abs(mean - mu) < 5 * np.sqrt(var / n))
    assert np.all(np.abs(v / var - 1) < 6 * np.sqrt(2.0 / n) + 1e-3)


@pytest.mark.parametrize("camera", [0, 2], ids=["poisson", "scmos-adu"])
@pytest.mark.parametrize("case", CASES[:4], ids=[c[0] for c in CASES[:4]])
def test_fits_of_generated_rois_reach_the_crlb(ctx, case, camera):
    """Fits of 20 000 generated copies of one emitter: x and y unbiased within
    0.05 px and their spread within 10% (Poisson) or 30% (sCMOS) of the mean
    CRLB."""
    torch = pytest.importorskip("torch")
    name, model, box = case
    w = make_case(name, model, box, 2, 4, seed=13)
    _maps(ctx, w.maps)
    n = 20_000
    theta = {0: [5.8, 6.3, 2000, 10], 1: [4.8, 5.3, 2000, 10, 1.4],
             2: [6.8, 7.3, 2000, 10, 1.3, 1.7], 3: [7.9, 8.2, 120, 3000, 10]}[model]
    truth = np.tile(np.array(theta, np.float32), (n, 1))
    rng = np.random.default_rng(3)
    xc = rng.integers(1, 256 - box + 2, n).astype(np.int32)
    yc = rng.integers(1, 256 - box + 2, n).astype(np.int32)
    data = _gen(torch, ctx, w, camera, truth, 2024 + model, xc, yc)
    P = w.psf.nparams
    dev = torch.device("cuda", 0)
    d = torch.from_numpy(np.ascontiguousarray(data.transpose(2, 1, 0)).reshape(-1)).to(dev)
    params = torch.empty((n, P), device=dev)
    crlb = torch.empty((n, P), device=dev)
    llr = torch.empty(n, device=dev)
    flags = torch.empty(n, dtype=torch.uint8, device=dev)
    G.fit_device(ctx, make_desc(w.psf, box, 20, w.constraints, camera), d,
                 torch.from_numpy(xc).to(dev), torch.from_numpy(yc).to(dev), params, crlb, llr,
                 flags)
    torch.cuda.synchronize()
    prm, cr, fl = params.cpu().numpy(), crlb.cpu().numpy(), flags.cpu().numpy()
    ok = (fl & 1).astype(bool)
    assert ok.mean() > 0.99
    for k in (0, 1):
        est, err = prm[ok, k], cr[ok, k]
        assert abs(est.mean() - theta[k]) < 0.05
        bar = 0.10 if camera == 0 else 0.30
        assert abs(est.std() / err.mean() - 1) < bar, (k, est.std(), err.mean())
