"""ctypes binding of libgaussmle_sm100a.so (include/gaussmle_gb300.h).

This is the Python twin of the Julia `ccall` shim: the same C entry points,
argument meanings and status codes.  Loading fails loudly when the library is
missing - there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

GMLE_OK = 0
STATUS_NAMES = {
    0: "GMLE_OK", 1: "GMLE_INVALID_ARG", 2: "GMLE_UNSUPPORTED_MODEL", 3: "GMLE_UNSUPPORTED_BOX",
    4: "GMLE_OUT_OF_MEMORY", 5: "GMLE_ADMISSION_REJECTED", 6: "GMLE_CUDA_ERROR",
    7: "GMLE_TIMEOUT", 8: "GMLE_NO_DEVICE", 9: "GMLE_NOT_READY",
}

FLAG_CONVERGED = 1
FLAG_CHOLESKY = 2
FLAG_LU = 4
FLAG_SINGULAR = 8

CAMERA_POISSON = 0
CAMERA_SCMOS = 1
CAMERA_SCMOS_ADU = 2

# Every symbol the header declares (checked by the CPU test-suite).
EXPORTED = [
    "gmle_abi_version", "gmle_create", "gmle_destroy", "gmle_last_error",
    "gmle_set_calibration", "gmle_fit", "gmle_fit_device", "gmle_fit_device_errors",
    "gmle_get_tuning", "gmle_set_tuning", "gmle_autotune", "gmle_kernel_launches",
    "gmle_fit_mixed_device", "gmle_server_start", "gmle_server_stop", "gmle_submit",
    "gmle_submit_many",
    "gmle_poll", "gmle_wait", "gmle_server_stats_get", "gmle_fit_mixed_device_noalloc",
    "gmle_pvalues", "gmle_pvalues_device", "gmle_cut_rois_device", "gmle_simulate_device",
    "gmle_math_selftest",
]


class FitDesc(C.Structure):
    """gmle_fit_desc: the non-array arguments of unified_gaussian_mle_kernel!
    (src/unified_kernel.jl:286-297)."""
    _fields_ = [
        ("model", C.c_int32), ("box", C.c_int32), ("iterations", C.c_int32),
        ("camera", C.c_int32), ("psf", C.c_float * 8), ("lower", C.c_float * 6),
        ("upper", C.c_float * 6), ("max_step", C.c_float * 6), ("method", C.c_int32),
    ]


METHOD_NEWTON, METHOD_FISHER_LM = 0, 1


class Group(C.Structure):
    """gmle_group: one homogeneous group of a mixed batch / one serving request."""
    _fields_ = [
        ("desc", FitDesc), ("data", C.c_void_p), ("x_corners", C.c_void_p),
        ("y_corners", C.c_void_p), ("n", C.c_int64), ("params", C.c_void_p),
        ("crlb", C.c_void_p), ("llr", C.c_void_p), ("flags", C.c_void_p),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("hbm_budget_bytes", C.c_int64), ("max_inflight_steps", C.c_int32),
        ("max_step_rois", C.c_int64), ("max_pending", C.c_int32), ("use_graphs", C.c_int32),
    ]


class ServerStats(C.Structure):
    _fields_ = [
        ("submitted", C.c_int64), ("completed", C.c_int64), ("rejected", C.c_int64),
        ("failed", C.c_int64), ("rois_completed", C.c_int64), ("steps", C.c_int64),
        ("p50_latency_ms", C.c_double), ("p99_latency_ms", C.c_double),
        ("mean_latency_ms", C.c_double), ("max_latency_ms", C.c_double),
        ("fits_per_s", C.c_double), ("hbm_budget_bytes", C.c_int64),
        ("hbm_in_use_bytes", C.c_int64), ("hbm_peak_bytes", C.c_int64),
    ]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class GaussMLEError(RuntimeError):
    """A non-zero gmle_status, with the context's gmle_last_error() message."""

    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


_lib = None
_lock = threading.Lock()


def library_path() -> Path:
    return _build.LIB_PATH


def load(path: str | Path | None = None) -> C.CDLL:
    """Load the library (building it first if the sources are newer)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else _build.LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build it with gaussmle_gb300.build.build() (needs nvcc)")
        lib = C.CDLL(str(p))
        vp, i32, i64, fp = C.c_void_p, C.c_int32, C.c_int64, C.c_void_p
        sigs = {
            "gmle_abi_version": ([], C.c_int),
            "gmle_create": ([C.POINTER(vp), C.c_int], C.c_int),
            "gmle_destroy": ([vp], None),
            "gmle_last_error": ([vp], C.c_char_p),
            "gmle_set_calibration": ([vp, fp, fp, fp, i32, i32], C.c_int),
            "gmle_fit": ([vp, C.POINTER(FitDesc), fp, fp, fp, i64, fp, fp, fp, fp], C.c_int),
            "gmle_fit_device": ([vp, C.POINTER(FitDesc), vp, vp, vp, i64, vp, vp, vp, vp, vp],
                                C.c_int),
            "gmle_fit_device_errors": ([vp, C.POINTER(i64)], C.c_int),
            "gmle_get_tuning": ([vp, i32, i32, i32, C.POINTER(i32), C.POINTER(i32)], C.c_int),
            "gmle_set_tuning": ([vp, i32, i32, i32, i32, i32], C.c_int),
            "gmle_autotune": ([vp, C.POINTER(FitDesc), vp, vp, vp, i64, vp, vp, vp, vp,
                               C.POINTER(i32), C.POINTER(i32), C.POINTER(C.c_float)], C.c_int),
            "gmle_kernel_launches": ([vp], i64),
            "gmle_fit_mixed_device": ([vp, C.POINTER(Group), i32, vp], C.c_int),
            "gmle_server_start": ([vp, C.POINTER(ServerConfig)], C.c_int),
            "gmle_server_stop": ([vp], C.c_int),
            "gmle_submit": ([vp, C.POINTER(Group), C.POINTER(C.c_uint64)], C.c_int),
            "gmle_submit_many": ([vp, C.POINTER(Group), C.c_int32, C.POINTER(C.c_uint64),
                                  C.POINTER(C.c_int32)], C.c_int),
            "gmle_poll": ([vp, C.c_uint64], C.c_int),
            "gmle_wait": ([vp, C.c_uint64, i64], C.c_int),
            "gmle_server_stats_get": ([vp, C.POINTER(ServerStats), i32], C.c_int),
            "gmle_pvalues": ([vp, fp, i64, i32, fp], C.c_int),
            "gmle_cut_rois_device": ([vp, vp, i32, i32, i64, vp, vp, vp, i64, i32, vp, vp],
                                     C.c_int),
            "gmle_pvalues_device": ([vp, vp, i64, i32, vp, vp], C.c_int),
            "gmle_simulate_device": ([vp, vp, vp, vp, vp, i64, C.c_uint64, vp, vp], C.c_int),
            "gmle_fit_mixed_device_noalloc": ([C.POINTER(Group), i32, vp, vp, vp, i32, i32, vp,
                                               C.c_char_p, i32], C.c_int),
            "gmle_math_selftest": ([vp, i64, vp, vp], C.c_int),
        }
        for name, (args, res) in sigs.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _lib = lib
        return lib


def check(lib: C.CDLL, ctx, status: int) -> None:
    if status != GMLE_OK:
        msg = lib.gmle_last_error(ctx) if ctx else b""
        raise GaussMLEError(status, (msg or b"").decode(errors="replace"))


class Context:
    """Owns one gmle_ctx (device streams, resident calibration maps, buffers)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        self._ctx = C.c_void_p()
        st = self.lib.gmle_create(C.byref(self._ctx), device)
        if st != GMLE_OK:
            raise GaussMLEError(st, f"cannot create a context on CUDA device {device} "
                                    "(a GB300 / sm_103a device is required; no CPU fallback)")
        self.device = device

    @property
    def handle(self):
        return self._ctx

    def close(self) -> None:
        if self._ctx:
            self.lib.gmle_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, status: int) -> None:
        check(self.lib, self._ctx, status)

    def launches(self) -> int:
        return int(self.lib.gmle_kernel_launches(self._ctx))


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx
