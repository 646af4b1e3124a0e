"""Build libgaussmle_sm100a.so in-tree with nvcc for sm_103a.

The library is the product: eight kernel translation units (PSF model x camera
family) plus the C-ABI runtime, compiled in parallel (one -gencode, no cmake;
the heaviest units first) and linked into ``<package root>/lib/libgaussmle_sm100a.so``.
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
SOURCES = [f"gmle_fit_{m}_{cam}.cu" for m in ("astig", "xynbsxsy", "xynbs", "xynb")
           for cam in ("poisson", "scmos")] + ["gmle_runtime.cu", "gmle_server.cu",
                                                "gmle_noalloc.cu", "gmle_pvalue.cu",
                                                "gmle_frames.cu", "gmle_simulate.cu"]


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


def _compile(src: str, verbose: bool) -> Path:
    obj = BUILD_DIR / (Path(src).stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(res.stderr)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile the CUDA library if any source is newer than it; return its path."""
    if not force and up_to_date():
        return LIB_PATH
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    workers = min(len(SOURCES), os.cpu_count() or 1)
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
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
