"""Work and traffic per ROI: the one definition the benchmark's roofline uses.

The fit has no dense contraction, so the bound is the slower of
  (a) bytes in and out over HBM bandwidth, and
  (b) the per-ROI FP32-pipe + SFU (MUFU) instruction count at their peak rates.
Counts are for the *separable minimum* algorithm (per Newton iteration, the
erf/exp terms are evaluated once per pixel index and axis, not per pixel),
which is stricter than the reference's per-pixel recomputation
(src/psf_derivatives.jl calls 4 erf + 4 exp per pixel per iteration).

Instruction cost table (lane instructions; a minimum implementation):
  erf        1 SFU + 10 FP32   (polynomial/rational core + one exp2)
  exp        1 SFU +  2 FP32   (scale by log2 e, ex2)
  log        1 SFU +  2 FP32
  div, rcp   1 SFU +  2 FP32   (reciprocal + one refinement/multiply)
  sqrt       1 SFU +  1 FP32
  add/mul/fma/min/compare/select: 1 FP32
FP64 work (Fisher accumulation per column, inversion) is listed separately
and converted at GB300's FP64:FP32 rate (1/64) into FP32 issue slots.
SFU instructions are converted at the MUFU:FP32 lane ratio of an SM
(16 : 128) into FP32 issue slots, so one number ("FP32-equivalent
instructions") measures the issue-bound work.
"""
from __future__ import annotations

SFU_RATIO = 8.0     # FP32 lanes per MUFU lane in one SM (128 / 16)
FP64_RATIO = 64.0   # FP32 / FP64 throughput on GB300

NPARAMS = {0: 4, 1: 5, 2: 6, 3: 5}


def _cost(erf=0, exp=0, log=0, div=0, sqrt=0, fp32=0):
    sfu = erf + exp + log + div + sqrt
    f = 10 * erf + 2 * exp + 2 * log + 2 * div + 1 * sqrt + fp32
    return f, sfu


def work_per_roi(model: int, box: int, iterations: int = 20, camera: int = 0) -> dict:
    """Instruction counts of one ROI fit (see the module docstring)."""
    P = NPARAMS[model]
    sig = model != 0
    scmos = camera != 0
    # per axis entry: 2 erf, 2 exp, 2 div (argument scaling), ~12 FP32 arithmetic;
    # sigma models add the two sigma-derivative products (~10 FP32)
    ent_f, ent_s = _cost(erf=2, exp=2, div=2, fp32=12 + (10 if sig else 0))
    # per pixel and iteration: model value, likelihood terms (one reciprocal),
    # dudt / d2udt2 products, gradient and Hessian accumulation
    dudt = {0: 5, 1: 11, 2: 11, 3: 15}[model]
    acc = 2 * P + 3 * (2 + (1 if model == 1 else 0) + (2 if model == 2 else 0) +
                       (1 if model == 3 else 0))
    px_f, px_s = _cost(div=1, fp32=1 + (3 if scmos else 5) + dudt + acc)
    per_iter_f = 2 * box * ent_f + box * box * px_f + 40  # + Newton update
    per_iter_s = 2 * box * ent_s + box * box * px_s
    # final pass: tables again, LLR (Poisson: 2 log; sCMOS: 1 div), Fisher products
    fis = P + P * (P + 1) // 2
    fin_f, fin_s = _cost(log=0 if scmos else 2, div=2, fp32=8 + dudt + fis)
    final_f = 2 * box * ent_f + box * box * fin_f
    final_s = 2 * box * ent_s + box * box * fin_s
    init_f = 3 * box * box + 40
    fp32 = iterations * per_iter_f + final_f + init_f
    sfu = iterations * per_iter_s + final_s
    # FP64: per-column Fisher accumulation + Cholesky/inverse (~P^3/2 + 10P ops)
    fp64 = box * P * (P + 1) // 2 + P ** 3 // 2 + 10 * P
    equiv = fp32 + SFU_RATIO * sfu + FP64_RATIO * fp64
    return {"fp32": fp32, "sfu": sfu, "fp64": fp64, "fp32_equiv": equiv}


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
