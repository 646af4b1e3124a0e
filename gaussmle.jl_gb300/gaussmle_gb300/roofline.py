"""Work and traffic per ROI: the one definition the benchmark's roofline uses.

The fit has no dense contraction, so the bound is the slower of
  (a) bytes in and out over HBM bandwidth, and
  (b) the per-ROI FP32 + SFU (MUFU) + FP64 instruction count at peak,
with SFU and FP64 instructions converted into FP32 issue slots by the lane
ratios of a GB300 SM (MUFU 16 : FP32 128 lanes per clock -> 8 slots; FP64
about 2 : 128 -> 64 slots), i.e. as if the pipes did not overlap.

Counts follow the minimum of the algorithm the kernel implements, which is
already far below the reference's per-pixel recomputation
(src/psf_derivatives.jl: 4 erf + 4 exp + ~60 FP32 per pixel per iteration):
  * per Newton iteration and axis, one table entry per pixel index with the
    erf/exp of shared pixel edges evaluated once (1 erf + 1 exp per entry);
  * per pixel, the model value, the likelihood terms (one reciprocal) and 6-7
    running sums (the gradient and diagonal Hessian are separable sums);
  * per column / row, the table factors applied to those sums;
  * final pass: LLR terms, Fisher weight sums, FP64 accumulation and the FP64
    Cholesky inversion.
Instruction cost table (lane instructions):
  erf 1 SFU + 10 FP32;  exp, log 1 SFU + 2 FP32;  reciprocal 1 SFU + 1 FP32;
  IEEE division 1 SFU + 7 FP32;  sqrt 1 SFU + 1 FP32;
  add / mul / fma / min / compare / select: 1 FP32.
Loads, stores, integer and control instructions are not counted.
"""
from __future__ import annotations

SFU_SLOTS = 8.0     # FP32 lanes per MUFU lane in one SM (128 / 16)
FP64_SLOTS = 64.0   # FP32 / FP64 throughput on GB300

NPARAMS = {0: 4, 1: 5, 2: 6, 3: 5}


def _c(erf=0, exp=0, log=0, rcp=0, div=0, sqrt=0, fp32=0):
    """(FP32, SFU) lane instructions of a bundle of operations."""
    sfu = erf + exp + log + rcp + div + sqrt
    f = 10 * erf + 2 * exp + 2 * log + rcp + 7 * div + sqrt + fp32
    return f, sfu


def work_per_roi(model: int, box: int, iterations: int = 20, camera: int = 0) -> dict:
    """Lane-instruction counts of one ROI fit (see the module docstring)."""
    P = NPARAMS[model]
    sig = model != 0
    scmos = camera != 0
    cross = model in (1, 3)

    def add(acc, x, k=1):
        acc[0] += k * x[0]
        acc[1] += k * x[1]

    it = [0, 0]
    # axis set-up (one IEEE division, ~10 products) x 2 axes; astigmatic widths
    add(it, _c(div=2, fp32=20 + (60 if model == 3 else 0)))
    # table entries: 1 erf + 1 exp + arithmetic (second derivatives included)
    add(it, _c(erf=1, exp=1, fp32=16 + (10 if sig else 0)), 2 * box)
    # pixels: mu, likelihood terms, running sums
    lik = _c(rcp=1, fp32=3) if scmos else _c(rcp=1, fp32=7)
    add(it, (1 + lik[0] + 6 + (1 if cross else 0), lik[1]), box * box)
    # per column and per row: table factors applied to the sums
    add(it, (2 + 8 + {0: 0, 1: 8, 2: 5, 3: 12}[model], 0), box)
    add(it, (4 + {0: 0, 1: 5, 2: 5, 3: 8}[model], 0), box)
    # Newton step: one IEEE division and two clamps per parameter
    add(it, _c(div=1, fp32=6), P)

    fin = [0, 0]
    add(fin, _c(div=2, fp32=20 + (60 if model == 3 else 0)))
    add(fin, _c(erf=1, exp=1, fp32=10 + (4 if sig else 0)), 2 * box)
    llr = _c(div=1, fp32=4) if scmos else _c(log=2, fp32=6)
    nq = 10 if sig else 6
    add(fin, (1 + llr[0] + 3 + nq + (3 if sig else 2), llr[1] + 1), box * box)
    terms = P * (P + 1) // 2 + (P if cross else 0)
    add(fin, (2 * terms, 0), box)
    # FP64: per-column accumulation and Cholesky / inverse / CRLB
    fp64 = box * P * (P + 1) // 2 + (P ** 3) // 3 + 2 * P * P + 12 * P
    init = 3 * box * box + 40
    fp32 = iterations * it[0] + fin[0] + init
    sfu = iterations * it[1] + fin[1]
    return {"fp32": fp32, "sfu": sfu, "fp64": fp64,
            "fp32_equiv": fp32 + SFU_SLOTS * sfu + FP64_SLOTS * fp64,
            "issue": fp32 + sfu + fp64}


def bytes_per_roi(model: int, box: int, camera: int = 0, flags: bool = True) -> int:
    """Algorithmic HBM bytes of one ROI: pixels in (+ the calibration tile for
    sCMOS: variance, and gain + offset for ADU data), corners, outputs."""
    P = NPARAMS[model]
    b2 = box * box
    inp = 4 * b2 + 8
    if camera == 1:
        inp += 4 * b2
    elif camera == 2:
        inp += 12 * b2
    out = 8 * P + 4 + (1 if flags else 0)
    return inp + out
