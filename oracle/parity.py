"""Parity bar and comparison of fit results against the oracle.

TEST INFRASTRUCTURE ONLY: used by tests/ and by the CPU-baseline leg of
bench.py to compare the CUDA path's outputs with the oracle's on the same
ROIs.  The product path never imports it.

The bar (the tolerances asked of the rebuilt fit against the reference's CPU
path on identical inputs, the same ones test/gpu_tests.jl:224-226 applies
between the reference's CPU and GPU back ends, tightened):
  positions, sigmas and z within 1e-3 (pixels, or the units of gamma and d),
  N and bg within 1e-4 relative, CRLB within 1e-3 relative, and the same
  convergence flag (isfinite(CRLB_x)).
"""
from __future__ import annotations

import numpy as np

TOL_POS = 1e-3
TOL_REL_NBG = 1e-4
TOL_REL_CRLB = 1e-3

# parameter slots per model: positions / widths / z, then N and bg
POS_SLOTS = {0: [0, 1], 1: [0, 1, 4], 2: [0, 1, 4, 5], 3: [0, 1, 2]}
NBG_SLOTS = {0: [2, 3], 1: [2, 3], 2: [2, 3], 3: [3, 4]}


def distance(model: int, params: np.ndarray, ref_params: np.ndarray) -> np.ndarray:
    """Per-ROI distance of params from ref_params in units of the bar: the
    largest of |d pos| / 1e-3 and |d N|, |d bg| relative / 1e-4 (<= 1 passes)."""
    p, r = params.astype(np.float64), ref_params.astype(np.float64)
    dpos = np.abs(p[:, POS_SLOTS[model]] - r[:, POS_SLOTS[model]]).max(1) / TOL_POS
    inb = NBG_SLOTS[model]
    dnb = (np.abs(p[:, inb] - r[:, inb]) / np.maximum(np.abs(r[:, inb]), 1e-30)).max(1)
    return np.maximum(dpos, dnb / TOL_REL_NBG)


def crlb_rel(crlb: np.ndarray, ref_crlb: np.ndarray) -> np.ndarray:
    """Per-ROI largest relative CRLB difference; 0 where both are non-finite
    alike, inf where exactly one is finite."""
    c, r = crlb.astype(np.float64), ref_crlb.astype(np.float64)
    fin = np.isfinite(r) & np.isfinite(c)
    d = np.where(fin, np.abs(c - r) / np.maximum(np.abs(r), 1e-30), 0.0)
    return np.where(np.isfinite(r) == np.isfinite(c), d, np.inf).max(1)


def compare(model, got_params, got_crlb, got_flags, ref):
    """Per-ROI pass mask and the largest errors against the oracle outputs."""
    rp, gp = ref["params"].astype(np.float64), got_params.astype(np.float64)
    dpos = np.abs(gp[:, POS_SLOTS[model]] - rp[:, POS_SLOTS[model]]).max(1)
    inb = NBG_SLOTS[model]
    dnb = (np.abs(gp[:, inb] - rp[:, inb]) / np.maximum(np.abs(rp[:, inb]), 1e-30)).max(1)
    dcr = crlb_rel(got_crlb, ref["crlb"])
    same_flag = (got_flags & 1) == (ref["flags"] & 1)
    ok = (dpos <= TOL_POS) & (dnb <= TOL_REL_NBG) & (dcr <= TOL_REL_CRLB) & same_flag
    return ok, {"max_dpos": float(dpos.max()), "max_rel_nbg": float(dnb.max()),
                "max_rel_crlb": float(dcr.max()), "flag_mismatch": int((~same_flag).sum()),
                "pass_frac": float(ok.mean())}


def _q(x, q):
    x = x[np.isfinite(x)]
    return float(np.quantile(x, q)) if x.size else None


def group_report(model, gpu: dict, f32: dict, f64: dict | None = None,
                 f64_sel: np.ndarray | None = None, gpu_final64: dict | None = None,
                 f32_final64: dict | None = None) -> dict:
    """Parity of one (model, box, camera) group of ROIs.

    gpu, f32: outputs (params, crlb, llr, flags) of the CUDA path and of the
    FP32 oracle on the same ROIs.  f64: the FP64 oracle on the subset f64_sel
    (indices into those ROIs).  gpu_final64 / f32_final64: the FP64 final pass
    at the GPU's / the FP32 oracle's own fitted parameters, on that subset.

    Reported: the pass fraction and largest errors against the FP32 oracle;
    for each ROI that misses the bar, whether the FP32 oracle itself is off
    the FP64 oracle by more than the bar (the iteration is unstable there) and
    whether the GPU is at least as close to the FP64 oracle; the distance of
    both to the FP64 oracle; and the CRLB error of each against the FP64 final
    pass at its own parameters (the error of the Fisher accumulation and
    inversion alone)."""
    ok, st = compare(model, gpu["params"], gpu["crlb"], gpu["flags"], f32)
    llr_rel = np.abs(gpu["llr"].astype(np.float64) - f32["llr"]) / \
        np.maximum(np.abs(f32["llr"].astype(np.float64)), 1e-6)
    st["n"] = int(len(ok))
    st["misses"] = int((~ok).sum())
    st["llr_rel_p99"] = _q(llr_rel, 0.99)
    if f64 is not None:
        sel = np.arange(len(ok)) if f64_sel is None else np.asarray(f64_sel)
        g_p, f_p = gpu["params"][sel], f32["params"][sel]
        d_gpu = distance(model, g_p, f64["params"])
        d_f32 = distance(model, f_p, f64["params"])
        miss = ~ok[sel]
        st["fp64"] = {
            "n": int(len(sel)),
            "gpu_dist_p50": _q(d_gpu, 0.5), "gpu_dist_p99": _q(d_gpu, 0.99),
            "f32_dist_p50": _q(d_f32, 0.5), "f32_dist_p99": _q(d_f32, 0.99),
            "gpu_within_bar_frac": float((d_gpu <= 1).mean()),
            "f32_within_bar_frac": float((d_f32 <= 1).mean()),
            "gpu_crlb_rel_p99": _q(crlb_rel(gpu["crlb"][sel], f64["crlb"]), 0.99),
            "f32_crlb_rel_p99": _q(crlb_rel(f32["crlb"][sel], f64["crlb"]), 0.99),
            "misses": int(miss.sum()),
            # a miss is explained when the FP32 path is itself off the exact
            # (FP64) iteration by more than the bar, with the GPU no farther
            "misses_f32_off_bar": int((miss & (d_f32 > 1)).sum()),
            "misses_gpu_no_farther": int((miss & (d_gpu <= d_f32)).sum()),
            "misses_explained": int((miss & (d_f32 > 1) & (d_gpu <= d_f32)).sum()),
        }
        if gpu_final64 is not None:
            e_g = crlb_rel(gpu["crlb"][sel], gpu_final64["crlb"])
            st["fp64"]["gpu_crlb_vs_fp64_at_own_theta"] = {
                "p50": _q(e_g, 0.5), "p99": _q(e_g, 0.99), "max": _q(e_g, 1.0)}
        if f32_final64 is not None:
            e_f = crlb_rel(f32["crlb"][sel], f32_final64["crlb"])
            st["fp64"]["f32_crlb_vs_fp64_at_own_theta"] = {
                "p50": _q(e_f, 0.5), "p99": _q(e_f, 0.99), "max": _q(e_f, 1.0)}
    return st
