"""ctypes wrapper of the CPU oracle (oracle/gmle_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker.  The product path never uses it.
Parity with the reference itself is unpinned at the value level (the
reference is Julia, not runnable here, and ships no golden vectors); see the
header of gmle_oracle.c for what pins the oracle instead.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

FLAG_CONVERGED, FLAG_CHOLESKY, FLAG_LU, FLAG_SINGULAR = 1, 2, 4, 8


class OracleDesc(C.Structure):
    _fields_ = [
        ("model", C.c_int32), ("box", C.c_int32), ("iterations", C.c_int32),
        ("camera", C.c_int32), ("psf", C.c_float * 8), ("lower", C.c_float * 6),
        ("upper", C.c_float * 6), ("max_step", C.c_float * 6), ("method", C.c_int32),
    ]


def build(force: bool = False) -> Path:
    srcs = [HERE / "gmle_oracle.c", HERE / "gmle_oracle_body.h", HERE / "Makefile"]
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in srcs):
        subprocess.run(["make", "-s"] + (["-B"] if force else []) + ["-C", str(HERE)],
                       check=True, capture_output=True)
    return LIB


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        vp, i64 = C.c_void_p, C.c_int64
        for nm in ("oracle_fit_f32", "oracle_fit_f64"):
            f = getattr(L, nm)
            f.argtypes = [C.POINTER(OracleDesc), vp, vp, vp, i64, vp, vp, vp, C.c_int32,
                          C.c_int32, vp, vp, vp, vp, C.c_int]
            f.restype = C.c_int
        for nm in ("oracle_final_at_f32", "oracle_final_at_f64"):
            f = getattr(L, nm)
            f.argtypes = [C.POINTER(OracleDesc), vp, vp, vp, i64, vp, vp, vp, C.c_int32,
                          vp, vp, vp, vp, C.c_int]
            f.restype = C.c_int
        for nm in ("oracle_crlb_at_f32", "oracle_crlb_at_f64"):
            f = getattr(L, nm)
            f.argtypes = [C.c_int, C.c_int, vp, vp, vp]
            f.restype = C.c_int
        L.oracle_max_threads.restype = C.c_int
        _lib = L
    return _lib


def nparams(model: int) -> int:
    return 4 if model == 0 else (6 if model == 2 else 5)


def make_desc(model, box, iterations, camera, psf, lower, upper, max_step,
              method: int = 0) -> OracleDesc:
    d = OracleDesc()
    d.model, d.box, d.iterations, d.camera = model, box, iterations, camera
    d.method = method
    for t in range(8):
        d.psf[t] = float(psf[t])
    for k in range(len(lower)):
        d.lower[k] = float(lower[k])
        d.upper[k] = float(upper[k])
        d.max_step[k] = float(max_step[k])
    return d


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def fit(desc: OracleDesc, data: np.ndarray, xc=None, yc=None, maps=None,
        precision: str = "f32", threads: int = 0) -> dict:
    """Run the oracle over ROIs: data is (box, box, n) (any order; copied to
    Fortran order).  maps = (variance, gain, offset) (ny, nx) or None.
    Returns params/crlb (n, P), llr (n,), flags (n,)."""
    L = lib()
    data = np.asfortranarray(data, np.float32)
    n = data.shape[2]
    P = nparams(desc.model)
    dt = np.float32 if precision == "f32" else np.float64
    params = np.empty((n, P), dt)
    crlb = np.empty((n, P), dt)
    llr = np.empty(n, dt)
    flags = np.empty(n, np.uint8)
    var = gain = off = None
    ny = nx = 0
    if maps is not None:
        var, gain, off = (np.asfortranarray(m, np.float32) for m in maps)
        ny, nx = var.shape
    xc = None if xc is None else np.ascontiguousarray(xc, np.int32)
    yc = None if yc is None else np.ascontiguousarray(yc, np.int32)
    f = L.oracle_fit_f32 if precision == "f32" else L.oracle_fit_f64
    rc = f(C.byref(desc), _p(data), _p(xc), _p(yc), n, _p(var), _p(gain), _p(off), ny, nx,
           _p(params), _p(crlb), _p(llr), _p(flags), threads)
    if rc != 0:
        raise ValueError(f"oracle rejected the descriptor (code {rc})")
    return {"params": params, "crlb": crlb, "llr": llr, "flags": flags}


def final_at(desc: OracleDesc, data: np.ndarray, theta: np.ndarray, xc=None, yc=None,
             maps=None, precision: str = "f64", threads: int = 0) -> dict:
    """The reference's final pass (LLR, Fisher matrix, CRLB; src/unified_kernel.jl:354-431)
    of each ROI at the given parameters theta (n, P), without the Newton
    iterations: the error of another implementation's CRLB against this one,
    at that implementation's own theta, is the error of its Fisher
    accumulation and inversion alone.  Returns crlb (n, P), llr (n,), flags (n,)."""
    L = lib()
    data = np.asfortranarray(data, np.float32)
    n = data.shape[2]
    P = nparams(desc.model)
    th = np.ascontiguousarray(theta, np.float64).reshape(n, P)
    dt = np.float32 if precision == "f32" else np.float64
    crlb = np.empty((n, P), dt)
    llr = np.empty(n, dt)
    flags = np.empty(n, np.uint8)
    var = gain = off = None
    ny = 0
    if maps is not None:
        var, gain, off = (np.asfortranarray(m, np.float32) for m in maps)
        ny = var.shape[0]
    xc = None if xc is None else np.ascontiguousarray(xc, np.int32)
    yc = None if yc is None else np.ascontiguousarray(yc, np.int32)
    f = L.oracle_final_at_f32 if precision == "f32" else L.oracle_final_at_f64
    rc = f(C.byref(desc), _p(data), _p(xc), _p(yc), n, _p(var), _p(gain), _p(off), ny,
           _p(th), _p(crlb), _p(llr), _p(flags), threads)
    if rc != 0:
        raise ValueError(f"oracle rejected the descriptor (code {rc})")
    return {"crlb": crlb, "llr": llr, "flags": flags}


def crlb_at(model: int, box: int, psf, theta, precision: str = "f64"):
    """CRLB of the Poisson Fisher matrix at a fixed parameter vector."""
    L = lib()
    psf = np.asarray(psf, np.float32)
    th = np.asarray(theta, np.float64)
    P = nparams(model)
    out = np.empty(P, np.float32 if precision == "f32" else np.float64)
    f = L.oracle_crlb_at_f32 if precision == "f32" else L.oracle_crlb_at_f64
    flags = f(model, box, _p(psf), _p(th), _p(out))
    return out, flags


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def pvalues(llr: np.ndarray, df: int) -> np.ndarray:
    """The reference's goodness-of-fit p-values (src/interface.jl:265-275):
    chi2 = -2 llr in Float32, p = 1 - Float32(cdf(Chisq(df), chi2)), the cdf
    in Float64 with chi2 clamped at 0 (Distributions.jl / StatsFuns gammacdf).
    scipy's regularised incomplete gamma function stands in for
    SpecialFunctions.gamma_inc."""
    from scipy.special import gammainc
    chi2 = (np.float32(-2.0) * np.asarray(llr, np.float32)).astype(np.float64)
    cdf = gammainc(0.5 * df, 0.5 * np.maximum(chi2, 0.0))
    cdf = np.where(np.isnan(chi2), np.nan, cdf)
    return (np.float32(1.0) - cdf.astype(np.float32)).astype(np.float32)
