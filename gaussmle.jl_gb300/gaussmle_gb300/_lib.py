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
]


class FitDesc(C.Structure):
    """gmle_fit_desc: the non-array arguments of unified_gaussian_mle_kernel!
    (src/unified_kernel.jl:286-297)."""
    _fields_ = [
        ("model", C.c_int32), ("box", C.c_int32), ("iterations", C.c_int32),
        ("camera", C.c_int32), ("psf", C.c_float * 8), ("lower", C.c_float * 6),
        ("upper", C.c_float * 6), ("max_step", C.c_float * 6),
    ]


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
