"""Build libgaussmle_sm100a.so in-tree with nvcc for sm_103a.

The library is the product: the fit kernels, compiled from one family source
(csrc/gmle_fit_family.cu) as 24 units - per PSF model (4), camera family (2)
and part (3: one thread per ROI for the odd boxes 5..15, for the other boxes
3..16, several lanes per ROI) - plus the runtime-box kernel and the C-ABI
runtime, compiled in parallel (one -gencode, no cmake; the heaviest units
first) and linked into ``<package root>/lib/libgaussmle_sm100a.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent          # gaussmle.jl_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
BUILD_DIR = PKG_ROOT / "_build"
LIB_DIR = PKG_ROOT / "lib"
LIB_NAME = "libgaussmle_sm100a.so"
LIB_PATH = LIB_DIR / LIB_NAME

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
              f"-I{REPO_ROOT / 'include'}"]
# (source, object stem, extra flags); heaviest first: the one-thread parts of
# the astigmatic and sigma models
FAMILY = "gmle_fit_family.cu"
_NAMES = {0: "xynb", 1: "xynbs", 2: "xynbsxsy", 3: "astig"}
UNITS = [(FAMILY, f"gmle_fit_{_NAMES[m]}_{'scmos' if c else 'poisson'}_p{p}",
          [f"-DGMLE_MODEL={m}", f"-DGMLE_SCMOS={c}", f"-DGMLE_PART={p}"])
         for p in (0, 1, 2) for m in (3, 2, 1, 0) for c in (1, 0)] + \
        [(src, Path(src).stem, []) for src in
         ("gmle_fit_generic.cu", "gmle_runtime.cu", "gmle_server.cu", "gmle_noalloc.cu",
          "gmle_pvalue.cu", "gmle_frames.cu", "gmle_simulate.cu", "gmle_math.cu")]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path("/usr/local/cuda/bin/nvcc")
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cuh")) + \
        sorted((REPO_ROOT / "include").glob("*.h")) + [Path(__file__)]


def up_to_date() -> bool:
    if not LIB_PATH.exists():
        return False
    t = LIB_PATH.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _deps())


def _compile(unit, verbose: bool) -> Path:
    src, stem, defs = unit
    obj = BUILD_DIR / (stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *defs, "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {stem}:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(res.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the CUDA library if any source is newer than it; return its path."""
    if not force and up_to_date():
        return LIB_PATH
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    workers = min(len(UNITS), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda u: _compile(u, verbose), UNITS))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
