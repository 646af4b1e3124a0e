"""GPU parity on the benchmark workloads' own distributions and sizes.

* the XYNB 11x11 Poisson workload at its full 10 000 ROIs (seed 1000, the
  reference's CPU-runnable case);
* the mixed batch's five groups (sCMOS ADU on 2048x2048 maps, photons
  log-uniform 100..20000, so that the dim, clamp-prone fits near N = 100 are
  in every group), 25 000 ROIs;
* XYNBS 13x13 sCMOS ADU ROIs at random corners of 2048x2048 maps.

The CUDA path (through the C ABI) is compared with the FP32 oracle on the
same ROIs, and both with the FP64 oracle of the same iteration:
  * models 0-2: >= 99.5 % of ROIs within the bar;
  * the astigmatic model (z in +-400 with gamma = 50, d = 100: many fits are
    ill-posed, and clamped fixed-iteration Newton is discontinuous there, so
    an ulp can move a fit by more than the bar): >= 95 % within the bar, and
    the misses are the iteration's own instability, not the GPU's error:
    the GPU is within the bar of the exact (FP64) iteration on as many ROIs
    as the FP32 reference path is (to 1 % of the ROIs), and most misses
    (>= 60 %) are ROIs on which the FP32 path itself is off the FP64
    iteration by more than the bar;
  * the CRLB against the FP64 final pass at the GPU's own parameters (the
    error of its FP32 per-pixel terms, double-float accumulation and FP64
    inversion, without the iteration's) is within 1e-5 at the 99th
    percentile, or for the ill-conditioned astigmatic Fisher matrices at
    least 5 times closer than the FP32 reference path's CRLB is to the same
    pass at its own parameters (measured: 2.2e-5 against 2.8e-4).
The same comparison runs in the benchmark on the ROIs its CPU baseline fits.
"""
import numpy as np
import pytest

from gaussmle_gb300 import simulate
from oracle import oracle as O
from oracle import parity
from parity_cases import oracle_desc
from test_parity_gpu import run_gpu

pytestmark = pytest.mark.gpu

MIN_PASS = {0: 0.995, 1: 0.995, 2: 0.995, 3: 0.95}


def check(ctx, w, label):
    params, crlb, llr, flags = run_gpu(ctx, w)
    gpu = {"params": params, "crlb": crlb, "llr": llr, "flags": flags}
    d = oracle_desc(O, w)
    f32 = O.fit(d, w.data, w.x_corners, w.y_corners, w.maps, "f32")
    ok, _ = parity.compare(w.psf.model_id, params, crlb, flags, f32)
    sel = np.unique(np.concatenate([np.arange(min(w.n, 2000)), np.nonzero(~ok)[0]]))
    sub = w.data[:, :, sel]
    xc, yc = w.x_corners[sel], w.y_corners[sel]
    f64 = O.fit(d, sub, xc, yc, w.maps, "f64")
    gf = O.final_at(d, sub, params[sel], xc, yc, w.maps, "f64")
    ff = O.final_at(d, sub, f32["params"][sel], xc, yc, w.maps, "f64")
    st = parity.group_report(w.psf.model_id, gpu, f32, f64, sel, gf, ff)
    print(f"\n{label}: {st}")
    m = w.psf.model_id
    assert st["pass_frac"] >= MIN_PASS[m], st
    assert st["flag_mismatch"] <= max(1, int(1e-3 * w.n)), st
    f = st["fp64"]
    # as close to the exact (FP64) iteration as the FP32 reference path
    assert f["gpu_within_bar_frac"] >= f["f32_within_bar_frac"] - 0.01, st
    if m == 3 and f["misses"]:
        assert f["misses_f32_off_bar"] >= 0.6 * f["misses"], st
    g_own = st["fp64"]["gpu_crlb_vs_fp64_at_own_theta"]
    f_own = st["fp64"]["f32_crlb_vs_fp64_at_own_theta"]
    assert g_own["p99"] <= max(1e-5, 0.2 * f_own["p99"]), st
    assert g_own["max"] <= max(f_own["max"], 1e-5), st
    return st


def test_xynb11_poisson_full_10k(ctx):
    w = simulate.xynb11_poisson(n=10_000, seed=1000)
    check(ctx, w, "xynb-11-poisson 10 000 ROIs")


@pytest.fixture(scope="module")
def mixed():
    return simulate.mixed_batch_scmos(n=25_000, seed=1003)


@pytest.mark.parametrize("k", range(len(simulate.MIX)),
                         ids=[f"m{m}-{b}" for _, m, b in simulate.MIX])
def test_mixed_batch_groups(ctx, mixed, k):
    w = mixed[k]
    # the dim end of the photon range is present in every group
    n_true = w.truth[:, 3 if w.psf.model_id == 3 else 2]
    assert n_true.min() < 150
    check(ctx, w, f"mixed group {w.name} ({w.n} ROIs)")


def test_xynbs13_scmos_from_2048_maps(ctx):
    w = simulate.xynbs13_scmos(n=20_000, seed=1001)
    assert w.maps[0].shape == (2048, 2048)
    check(ctx, w, "xynbs-13-scmos-adu, 2048x2048 maps, 20 000 ROIs")
