"""Work and traffic per ROI: the one definition the benchmark's roofline uses.

The fit has no dense contraction, so no tensor-core peak applies.  Its bound
is the slowest of the resources one ROI uses, each at its peak:
  * HBM:  algorithmic bytes in and out / HBM bandwidth;
  * FP32: the FMA pipes take 128 FP32 lane operations per SM per clock
    (4 schedulers x 32 lanes).  A packed .f32x2 instruction issues two of
    them in one slot but still takes two lanes of the pipe, so the FP32
    operation count, not the instruction count, bounds the time;
  * SFU:  16 MUFU lanes per SM per clock, i.e. a MUFU operation holds its
    pipe for 8 FP32 slots;
  * FP64: about 2 lanes per SM per clock on GB300 (1/64 of FP32).
The pipes run concurrently, so the instruction bound of a ROI is
  max(fp32,  8 sfu,  64 fp64)   FP32 lane slots
(``work_per_roi()["slots"]``), and the roofline time of n ROIs is
  max(n bytes / HBM, n slots / FP32 peak).
Two labelled variants are kept beside it: ``issue`` = fp32 + sfu + fp64, the
issue slots the work takes when no FP32 operation is packed, and
``fp32_equiv_sum`` = fp32 + 8 sfu + 64 fp64, as if the pipes never overlapped.

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
Loads, stores, integer and control instructions are not counted: they are
the kernel's overhead, which the measured instruction count per ROI shows.
"""
from __future__ import annotations

SFU_SLOTS = 8.0     # FP32 lanes per MUFU lane in one SM (128 / 16)
FP64_SLOTS = 64.0   # FP32 / FP64 throughput on GB300
LANES_PER_SM = 128  # FP32 lane instructions issued per SM per clock

NPARAMS = {0: 4, 1: 5, 2: 6, 3: 5}


def _c(erf=0, exp=0, log=0, rcp=0, div=0, sqrt=0, fp32=0):
    """(FP32, SFU) lane instructions of a bundle of operations."""
    sfu = erf + exp + log + rcp + div + sqrt
    f = 10 * erf + 2 * exp + 2 * log + rcp + 7 * div + sqrt + fp32
    return f, sfu


def work_per_roi(model: int, box: int, iterations: int = 20, camera: int = 0) -> dict:
    """Lane-operation counts of one ROI fit (see the module docstring).

    Returns fp32, sfu, fp64 (lane operations), issue (= their sum: the issue
    slots without packing), slots (the overlapping-pipe bound in FP32 lane
    slots, the roofline's work) and fp32_equiv_sum (the non-overlapping
    variant)."""
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
    issue = fp32 + sfu + fp64
    return {"fp32": fp32, "sfu": sfu, "fp64": fp64, "issue": issue,
            "slots": max(fp32, SFU_SLOTS * sfu, FP64_SLOTS * fp64),
            "fp32_equiv_sum": fp32 + SFU_SLOTS * sfu + FP64_SLOTS * fp64}


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


def issue_peak_tinst(sm_count: int, sm_mhz: float) -> float:
    """FP32 peak of the GPU [T lane operations/s]: 128 per SM per clock (also
    the issue rate of unpacked lane instructions)."""
    return sm_count * LANES_PER_SM * sm_mhz * 1e6 / 1e12


def roofline(model: int, box: int, camera: int, n: int, seconds: float, sm_count: int,
             sm_mhz: float, hbm_gbs: float, iterations: int = 20) -> dict:
    """Roofline of one launch of n ROIs that took `seconds`: each resource's
    time at its peak, the bound (the largest), and the launch's fraction of it
    (bound time / measured time)."""
    w = work_per_roi(model, box, iterations, camera)
    b = bytes_per_roi(model, box, camera)
    peak = issue_peak_tinst(sm_count, sm_mhz)             # T FP32 lane slots/s
    t_fp32 = n * w["fp32"] / (peak * 1e12)
    t_sfu = n * w["sfu"] * SFU_SLOTS / (peak * 1e12)
    t_fp64 = n * w["fp64"] * FP64_SLOTS / (peak * 1e12)
    t_hbm = n * b / (hbm_gbs * 1e9)
    terms = {"fp32": t_fp32, "sfu": t_sfu, "fp64": t_fp64, "hbm": t_hbm}
    bound = max(terms, key=terms.get)
    return {"bound": bound, "frac": terms[bound] / seconds,
            "achieved_tinst": n * w["slots"] / seconds / 1e12, "peak_tinst": peak,
            "pipe_frac": {k: v / seconds for k, v in terms.items()},
            "issue_unpacked_frac": n * w["issue"] / (peak * 1e12) / seconds,
            "work": w, "bytes_per_roi": b}
