"""GPU parity: the CUDA fit (through the C ABI) against the FP32 oracle.

Bar: x, y, sigma, z within 1e-3; N, bg within 1e-4 relative; CRLB within 1e-3
relative; identical convergence flags (tests/parity_cases.py).  Each case also
states the error of both against the FP64 oracle of the same iteration.
"""
import ctypes as C

import numpy as np
import pytest

import gaussmle_gb300 as G
from gaussmle_gb300.fitter import make_desc
from oracle import oracle as O
from oracle import parity
from parity_cases import CASES, compare, make_case, oracle_desc

pytestmark = pytest.mark.gpu

# Fraction of ROIs that must meet every tolerance.  Fixed-iteration clamped
# Newton is discontinuous at the clamps: ulp-level differences (erf/exp
# implementations, FMA contraction, summation order) can flip a clamp for a
# fit that has not converged, so a small fraction may differ.  On the
# astigmatic cases the FP32 reference path itself is off the FP64 iteration
# by more than the bar on about 1 ROI in 50; the test checks below that the
# GPU is as close to the FP64 iteration as the FP32 path is.
MIN_PASS = {"astig-15-poisson": 0.97, "astig-15-scmos-adu": 0.97}
DEFAULT_MIN_PASS = 0.995


def run_gpu(ctx, w, iterations=20):
    P = w.psf.nparams
    desc = make_desc(w.psf, w.box, iterations, w.constraints, w.camera)
    if w.camera:
        var, gain, off = (np.asfortranarray(m) for m in w.maps)
        ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, var.ctypes.data_as(C.c_void_p),
                                               gain.ctypes.data_as(C.c_void_p),
                                               off.ctypes.data_as(C.c_void_p),
                                               var.shape[0], var.shape[1]))
    n = w.n
    params = np.empty((n, P), np.float32)
    crlb = np.empty((n, P), np.float32)
    llr = np.empty(n, np.float32)
    flags = np.empty(n, np.uint8)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    data = np.asfortranarray(w.data, np.float32)
    ctx.check(ctx.lib.gmle_fit(ctx.handle, C.byref(desc), p(data), p(w.x_corners),
                               p(w.y_corners), n, p(params), p(crlb), p(llr), p(flags)))
    return params, crlb, llr, flags


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_parity_vs_oracle(ctx, case):
    w = make_case(*case)
    params, crlb, llr, flags = run_gpu(ctx, w)
    ref = O.fit(oracle_desc(O, w), w.data, w.x_corners, w.y_corners, w.maps, "f32")
    ref64 = O.fit(oracle_desc(O, w), w.data, w.x_corners, w.y_corners, w.maps, "f64")
    ok, st = compare(w.psf.model_id, params, crlb, flags, ref)
    llr_rel = np.abs(llr - ref["llr"]) / np.maximum(np.abs(ref["llr"]), 1e-6)
    st["llr_rel_p99"] = float(np.quantile(llr_rel, 0.99))
    # error of each against the FP64 oracle of the same iteration
    e_gpu = np.abs(params - ref64["params"]).max(0)
    e_f32 = np.abs(ref["params"] - ref64["params"]).max(0)
    d_gpu = parity.distance(w.psf.model_id, params, ref64["params"])
    d_f32 = parity.distance(w.psf.model_id, ref["params"], ref64["params"])
    print(f"\n{w.name}: {st}\n  max|GPU-FP64| {e_gpu}\n  max|F32-FP64| {e_f32}"
          f"\n  within the bar of FP64: GPU {(d_gpu <= 1).mean():.4f}, "
          f"FP32 {(d_f32 <= 1).mean():.4f}")
    assert st["pass_frac"] >= MIN_PASS.get(w.name, DEFAULT_MIN_PASS), st
    # the GPU is as close to the exact (FP64) iteration as the FP32 reference
    # path is, to 1 % of the ROIs: the misses of the astigmatic cases are the
    # iteration's own sensitivity, shared by the FP32 path
    assert (d_gpu <= 1).mean() >= (d_f32 <= 1).mean() - 0.01
    assert np.quantile(llr_rel, 0.99) < 1e-4


def test_device_entry_matches_host_entry(ctx):
    torch = pytest.importorskip("torch")
    w = make_case("xynbs-13-scmos-adu", 1, 13, 2, 1500)
    hp, hc, hl, hf = run_gpu(ctx, w)
    dev = torch.device("cuda", 0)
    n, P = w.n, 5
    data = torch.from_numpy(np.ascontiguousarray(w.data.transpose(2, 1, 0)).reshape(-1)).to(dev)
    xc = torch.from_numpy(w.x_corners).to(dev)
    yc = torch.from_numpy(w.y_corners).to(dev)
    params = torch.empty((n, P), device=dev)
    crlb = torch.empty((n, P), device=dev)
    llr = torch.empty(n, device=dev)
    flags = torch.empty(n, dtype=torch.uint8, device=dev)
    desc = make_desc(w.psf, w.box, 20, w.constraints, w.camera)
    G.fit_device(ctx, desc, data, xc, yc, params, crlb, llr, flags)
    torch.cuda.synchronize()
    assert np.array_equal(params.cpu().numpy(), hp)
    assert np.array_equal(crlb.cpu().numpy(), hc)
    assert np.array_equal(flags.cpu().numpy(), hf)


SHAPE_CASES = [c for c in CASES if c[0] in ("xynb-11-poisson", "xynbs-13-scmos-adu",
                                           "xynbsxsy-13-scmos-adu", "astig-15-poisson")]


@pytest.mark.parametrize("tpr,rpb", [(1, 32), (1, 64), (1, 128), (4, 32), (4, 64), (8, 16),
                                     (8, 32)])
@pytest.mark.parametrize("case", SHAPE_CASES, ids=[c[0] for c in SHAPE_CASES])
def test_parity_every_launch_shape(ctx, case, tpr, rpb):
    """Both kernels (one thread per ROI, and lane groups of 4 and 8) meet the bar."""
    name, model, box, camera, n = case
    w = make_case(name, model, box, camera, min(n, 1500))
    ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, model, box, camera, tpr, rpb))
    try:
        params, crlb, llr, flags = run_gpu(ctx, w)
    finally:
        # (0, 0) removes the entry: back to the size-based default
        ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, model, box, camera, 0, 0))
    ref = O.fit(oracle_desc(O, w), w.data, w.x_corners, w.y_corners, w.maps, "f32")
    ok, st = compare(model, params, crlb, flags, ref)
    assert st["pass_frac"] >= MIN_PASS.get(w.name, DEFAULT_MIN_PASS), (tpr, rpb, st)
