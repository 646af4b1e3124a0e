"""CPU checks of the C ABI library: it builds, loads and exports every symbol
that include/gaussmle_gb300.h declares (no compute call needs a GPU here)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from gaussmle_gb300 import _lib, build

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "gaussmle_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(gmle_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return C.CDLL(str(build.LIB_PATH))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(_lib.EXPORTED)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_abi_version_and_no_device_error(lib):
    lib.gmle_abi_version.restype = C.c_int
    assert lib.gmle_abi_version() == 1
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present; the no-device path is not reachable")
    ctx = C.c_void_p()
    lib.gmle_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    st = lib.gmle_create(C.byref(ctx), 0)
    assert st == 8  # GMLE_NO_DEVICE: no CPU fallback
    assert not ctx


def test_fitdesc_layout_matches_header():
    # int32 x4 + float x (8 + 6 + 6 + 6) + int32 method
    assert C.sizeof(_lib.FitDesc) == 4 * 4 + 4 * 26 + 4
    assert _lib.FitDesc.psf.offset == 16 and _lib.FitDesc.lower.offset == 48
    assert _lib.FitDesc.upper.offset == 72 and _lib.FitDesc.max_step.offset == 96
    assert _lib.FitDesc.method.offset == 120


def test_fitter_without_gpu_raises():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import numpy as np
    import gaussmle_gb300 as G
    with pytest.raises(G.GaussMLEError):
        G.fit(G.GaussMLEFitter(), np.ones((7, 7, 2), np.float32))
    with pytest.raises(ValueError):
        G.GaussMLEFitter(device="cpu")
