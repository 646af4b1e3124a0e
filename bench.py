#!/usr/bin/env python3
"""Benchmark of the batched per-ROI Gaussian MLE fit on GB300.

Workload (default): GaussianXYNBS with fitted sigma (true sigma U(1.0, 1.8)),
13x13 Float32 ROIs, 1 000 000 ROIs per step, sCMOS camera with 2048x2048
device-resident variance / gain / offset maps, ADU data converted on the
device, 20 Newton iterations.  Synthetic, seeded data generated on the device.

One step = one fit of the whole batch.  `value` = ROI fits/s with the inputs
already in HBM (one kernel launch per step, CUDA events on the launch stream;
the 676 MB of pixel data per step exceed the 129 MB L2, so no flush is
needed).  `e2e` = the same metric through the C-ABI host-buffer call
gmle_fit() with pinned host buffers: H2D of pixels + corners and D2H of
params, CRLB, LLR and flags are inside the timed region.

`--impl reference` times the reference's algorithm on the host cores: the
FP32 CPU restatement of src/unified_kernel.jl (the reference is Julia, which
is not available here), OpenMP over ROIs on all host threads, each step a
bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "gaussmle.jl_gb300"))

import numpy as np  # noqa: E402

METRIC = "ROI fits/sec on 1 GB300 (plain one-launch-per-batch kernel)"
UNIT = "fits/s"
WORKLOAD = "gaussian-xynbs-13x13-scmos-1e6"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=1_000_000)
    p.add_argument("--cpu-seconds", type=float, default=10.0,
                   help="target CPU time of the cpu_baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--shape", default=None,
                   help="THREADS_PER_ROI,ROIS_PER_BLOCK: fixed launch shape instead of autotuning")
    return p.parse_args()


# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.idx = device_index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def fp32_peak_tinst(torch, dev) -> float:
    """Measured FP32 FFMA lane-instruction rate [T inst/s]: an FP32 SGEMM
    (TF32 off) issues 2 N^3 flops as N^3 FFMA lane instructions."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device=dev)
    b = torch.randn(n, n, device=dev)
    for _ in range(2):
        torch.mm(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.mm(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return n ** 3 / best / 1e12


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# ---------------------------------------------------------------------------

def cpu_baseline(wl_host: dict, seconds: float, threads: int = 0) -> dict:
    """Time the FP32 CPU restatement of the reference path on a bounded sample."""
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    from gaussmle_gb300.constraints import default_constraints
    from gaussmle_gb300.models import GaussianXYNBS
    cons = default_constraints(GaussianXYNBS(), 11)
    box = wl_host["box"]
    d = O.make_desc(1, box, 20, 2, np.zeros(8, np.float32), cons.lower, cons.upper,
                    cons.max_step)
    maps = wl_host["maps"]
    data = wl_host["data"]
    nth = threads if threads > 0 else O.max_threads()

    def run(m):
        t = time.perf_counter()
        O.fit(d, data[:, :, :m], wl_host["xc"][:m], wl_host["yc"][:m], maps, "f32", nth)
        return time.perf_counter() - t

    m0 = min(2000, data.shape[2])
    t0 = run(m0)
    m = int(min(data.shape[2], max(m0, m0 * seconds / max(t0, 1e-6))))
    t = run(m)
    return {"value": m / t, "unit": UNIT, "cores": nth, "kind": "port",
            "sample": f"first {m} ROIs of the workload ({t:.1f} s on {nth} host threads; "
                      "FP32 restatement of the reference CPU path, oracle/gmle_oracle.c)"}


def host_copy(wl: dict) -> dict:
    """Host (numpy) copies of the device workload for the CPU paths."""
    box, n = wl["box"], wl["n"]
    data = wl["data"].cpu().numpy().reshape(n, box, box).transpose(2, 1, 0)
    var = wl["var"].cpu().numpy().T
    gain = wl["gain"].cpu().numpy().T
    off = wl["offset"].cpu().numpy().T
    return {"data": data, "xc": wl["xc"].cpu().numpy(), "yc": wl["yc"].cpu().numpy(),
            "maps": (var, gain, off), "box": box, "n": n}


# ---------------------------------------------------------------------------

def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, local = dist_init()
    if rank != 0:
        return
    import torch
    from gaussmle_gb300 import simulate
    dev = "cuda:0" if torch.cuda.is_available() else "cpu"
    wl = simulate.config1_device(n=min(args.n, 200_000), device=dev)
    host = host_copy(wl)
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    from gaussmle_gb300.constraints import default_constraints
    from gaussmle_gb300.models import GaussianXYNBS
    cons = default_constraints(GaussianXYNBS(), 11)
    d = O.make_desc(1, 13, 20, 2, np.zeros(8, np.float32), cons.lower, cons.upper, cons.max_step)
    nth = O.max_threads()
    per_step = 20_000
    data = host["data"]

    def step(k):
        lo = (k * per_step) % (data.shape[2] - per_step)
        O.fit(d, data[:, :, lo:lo + per_step], host["xc"][lo:lo + per_step],
              host["yc"][lo:lo + per_step], host["maps"], "f32", nth)

    for k in range(args.warmup):
        step(k)
    t = time.perf_counter()
    for k in range(args.steps):
        step(args.warmup + k)
    dt = time.perf_counter() - t
    value = per_step * args.steps / dt
    sample = (f"{per_step} ROIs of the workload per step on {nth} host threads "
              "(FP32 restatement of the reference CPU path, oracle/gmle_oracle.c; "
              "the Julia reference is not installable here)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rois_per_step": per_step, "iterations": 20},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def run_ours(args):
    import torch
    world, rank, local = dist_init()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import gaussmle_gb300 as G
    from gaussmle_gb300 import simulate, roofline
    from gaussmle_gb300.fitter import make_desc

    n = args.n
    wl = simulate.config1_device(n=n, seed=1001 + rank, device=dev)
    ctx = G.Context(local)
    desc = make_desc(G.GaussianXYNBS(), 13, 20, G.default_constraints(G.GaussianXYNBS(), 11), 2)
    # calibration maps: device-resident, uploaded once
    var_h, gain_h, off_h = (wl[k].cpu().numpy() for k in ("var", "gain", "offset"))
    ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, var_h.ctypes.data_as(C.c_void_p),
                                           gain_h.ctypes.data_as(C.c_void_p),
                                           off_h.ctypes.data_as(C.c_void_p), wl["ny"], wl["nx"]))
    P = 5
    params = torch.empty((n, P), device=dev)
    crlb = torch.empty((n, P), device=dev)
    llr = torch.empty(n, device=dev)
    flags = torch.empty(n, dtype=torch.uint8, device=dev)
    stream = torch.cuda.Stream(dev)   # the launch stream; events are recorded on it

    def step():
        G.fit_device(ctx, desc, wl["data"], wl["xc"], wl["yc"], params, crlb, llr, flags,
                     stream=stream)

    # launch shape chosen by the project's autotuner (untimed), or fixed by --shape
    from gaussmle_gb300 import tuning
    if args.shape:
        tpr, rpb = (int(v) for v in args.shape.split(","))
        ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, 1, 13, 2, tpr, rpb))
        tune = (tpr, rpb, None)
    else:
        tune = tuning.autotune(ctx, desc, wl["data"], wl["xc"], wl["yc"], params, crlb, llr,
                               flags, save=False)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    # time of one launch alone (for the roofline; same stream, events around it)
    a0 = torch.cuda.Event(enable_timing=True)
    a1 = torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    step()
    a1.record(stream)
    torch.cuda.synchronize()
    single_launch_s = a0.elapsed_time(a1) / 1e3
    launches0 = ctx.launches()
    sampler = ClockSampler(local)
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    dt = e0.elapsed_time(e1) / 1e3
    if world > 1:
        t = torch.tensor([dt], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dt = float(t.item())
        dist.barrier()
    launches = ctx.launches() - launches0
    value = n * args.steps * world / dt
    per_launch = dt / args.steps
    conv = float((flags.cpu().numpy() & 1).mean())

    # ---- end to end through the C-ABI host-buffer call (pinned host memory) ----
    e2e = None
    if not args.no_e2e:
        h_data = wl["data"].cpu().pin_memory()
        h_xc = wl["xc"].cpu().pin_memory()
        h_yc = wl["yc"].cpu().pin_memory()
        h_par = torch.empty((n, P), pin_memory=True)
        h_crlb = torch.empty((n, P), pin_memory=True)
        h_llr = torch.empty(n, pin_memory=True)
        h_fl = torch.empty(n, dtype=torch.uint8, pin_memory=True)
        vp = lambda t: C.c_void_p(t.data_ptr())

        def host_step():
            ctx.check(ctx.lib.gmle_fit(ctx.handle, C.byref(desc), vp(h_data), vp(h_xc), vp(h_yc),
                                       n, vp(h_par), vp(h_crlb), vp(h_llr), vp(h_fl)))
        for _ in range(max(args.warmup, 3)):
            host_step()
        l0 = ctx.launches()
        if world > 1:
            dist.barrier()
        t = time.perf_counter()
        for _ in range(args.steps):
            host_step()
        et = time.perf_counter() - t
        if world > 1:
            tt = torch.tensor([et], device=dev, dtype=torch.float64)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            et = float(tt.item())
        e2e = {"value": n * args.steps * world / et, "unit": UNIT,
               "h2d_bytes_per_step": n * (13 * 13 * 4 + 8),
               "d2h_bytes_per_step": n * (2 * P * 4 + 4 + 1),
               "gpu_launches": ctx.launches() - l0,
               "ms_per_step": et / args.steps * 1e3}

    if rank != 0:
        return
    # ---- roofline: issue-bound FP32 + SFU work vs the measured FP32 rate ----
    w = roofline.work_per_roi(1, 13, 20, 2)
    peak_inst = fp32_peak_tinst(torch, dev)  # T lane-inst/s
    achieved = w["fp32_equiv"] * n / per_launch / 1e12  # per launch, averaged over the K steps
    peaks = measured_peaks()
    bpr = roofline.bytes_per_roi(1, 13, 2)
    hbm_ach = bpr * n / per_launch / 1e9
    rl = {
        "bound": "fp32+sfu", "achieved": achieved, "peak": peak_inst, "unit": "Tinst/s",
        "frac": achieved / peak_inst, "traffic": None,
        "peak_source": "measured in this run: FP32 SGEMM 8192^3 (TF32 off) FFMA rate",
        "work_per_roi_fp32_equiv": w["fp32_equiv"], "single_launch_ms": single_launch_s * 1e3,
        "hbm": {"achieved_gbs": hbm_ach, "peak_gbs": peaks.get("hbm_gbs"),
                "frac": hbm_ach / peaks.get("hbm_gbs", 6800.0), "bytes_per_roi": bpr,
                "peak_source": "MEASURED_PEAKS.json" if "source" not in peaks else "fallback"},
    }
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(host_copy(wl), args.cpu_seconds)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_launch * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rois_per_step": n, "box": 13, "model": "GaussianXYNBS",
                   "camera": "sCMOS (ADU, device-side conversion)", "iterations": 20,
                   "parallelism": f"roi-shard x{world}", "l2": "inputs (676 MB/step) > L2",
                   "tuning": {"threads_per_roi": tune[0], "rois_per_block": tune[1],
                              "source": "--shape" if args.shape else "gmle_autotune"}},
        "gpu_launches": launches,
        "converged_fraction": conv,
        "clocks": clocks,
        "roofline": rl,
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
