#!/usr/bin/env python3
"""Benchmark of the batched per-ROI Gaussian MLE fit on GB300.

Workload: the mixed batch - 2 000 000 ROIs per step, 40% GaussianXYNB 11x11,
25% GaussianXYNBS 9x9, 15% GaussianXYNBSXSY 13x13, 15% AstigmaticXYZNB
15x15, 5% GaussianXYNB 7x7, photons log-uniform 100..20000, sCMOS ADU data
on device-resident 2048x2048 variance / gain / offset maps, 20 Newton
iterations.  Synthetic, seeded, generated on the device.

One step = one fit of the whole batch.
  value  ROI fits/s of the batch call gmle_fit_mixed_device (each group of
         >= 65536 ROIs in its own autotuned launch, smaller groups in one
         persistent table launch per kind) with the inputs resident in HBM;
         CUDA events on the launch stream; 1.4 GB of pixels per step exceed
         the 129 MB L2.
  roofline  the dominant kernel: each group's launch timed alone.
  e2e    the same batch through the serving API: cut into requests of
         log-uniform 50..50000 ROIs, submitted at once with pinned host
         buffers (gmle_submit), every H2D and D2H inside the timed region.
  plain  the same requests through the per-batch call gmle_fit, one at a
         time (the reference's one-launch-per-batch pattern), and the same
         batch as one plain launch per group on device-resident data.
  latency  p50/p99 of requests arriving as a Poisson process (served vs plain).
`--impl reference` times the reference algorithm on the host cores: the FP32
CPU restatement of src/unified_kernel.jl (the Julia reference is not
installable here), OpenMP over ROIs on all host threads, each step a bounded
sample of the same mixed batch.
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

METRIC = "ROI fits/sec on 1 GB300 (served mixed batch vs plain kernel); p50/p99 request latency"
UNIT = "fits/s"
WORKLOAD = ("mixed-batch: 40% XYNB 11x11, 25% XYNBS 9x9, 15% XYNBSXSY 13x13, "
            "15% astigmatic 15x15, 5% XYNB 7x7; sCMOS ADU, 2048x2048 maps; 20 iterations")

# DRAM bytes (read + write) per ROI of a launch, from one ncu capture of the
# kernel (dram__bytes_read.sum + dram__bytes_write.sum over the ROIs of the
# captured launch); the roofline's traffic scales it to the timed launch.
TRAFFIC_BYTES_PER_ROI: dict[str, float] = {
    # 90 000 ROIs, one thread per ROI, 128 ROIs/block (variances in tensor
    # memory, per-warp staging, packed pixel loop): 155.5 MB read + 5.2 MB written
    "fit_kernel_r1<3, 15, true, false>": 1785.3,
    # 240 000 ROIs, one thread per ROI, 128 ROIs/block (variances in tensor
    # memory, packed pixel loop): 195.7 MB read + 8.6 MB written
    "fit_kernel_r1<0, 11, true, false>": 851.4,
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=2_000_000, help="ROIs per step")
    p.add_argument("--cpu-seconds", type=float, default=10.0,
                   help="target CPU time of the cpu_baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-latency", action="store_true")
    p.add_argument("--no-extras", action="store_true")
    p.add_argument("--loads", default="1e6,5e6,2e7,5e7",
                   help="offered loads (ROIs/s) of the latency measurement")
    p.add_argument("--loads-10k", default="2e7,5e7",
                   help="offered loads (ROIs/s) of the 10 000-ROI request latency measurement")
    p.add_argument("--max-step-rois", type=int, default=0,
                   help="serving loop: ROIs per step (0: the library default)")
    p.add_argument("--max-inflight", type=int, default=0,
                   help="serving loop: concurrent steps (0: the library default)")
    p.add_argument("--server-graphs", type=int, default=0, choices=(0, 1),
                   help="serving loop: 1 replays a CUDA graph of persistent launches per "
                        "kind, 0 launches one block per tile directly")
    p.add_argument("--load-rois", type=float, default=2e7,
                   help="ROIs of arrivals per load point (bounded to about 1.5 s)")
    p.add_argument("--plain", default="",
                   help="MODEL,BOX,CAMERA,N: time only the plain launch of one homogeneous "
                        "device-resident workload (model 0..3, camera 0..2) and print its line")
    p.add_argument("--tpr", type=int, default=0,
                   help="with --plain: threads per ROI (0: the autotuner's choice)")
    p.add_argument("--rpb", type=int, default=0, help="with --plain: ROIs per block")
    p.add_argument("--method", default="newton", choices=["newton", "lm"],
                   help="with --plain: the reference's Newton step, or the full-Hessian option")
    return p.parse_args()


# ---------------------------------------------------------------------------

class ClockSampler:
    """SM clock, clock-event (throttle) reasons and power of the GPU, sampled
    every 5 ms through NVML (read-only queries) in a host thread; begin() and
    end() mark the timed region, and stop() summarises the samples inside it.
    Falls back to `nvidia-smi -lms 200` where NVML cannot be loaded."""
    # nvmlClocksEventReasons bits
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int, pci_bus_id: str | None = None):
        self.idx = device_index
        self.pci = pci_bus_id
        self.proc = None
        self.path = None
        self.nvml = None
        self.samples = []
        self.t0 = self.t1 = None

    def _open_nvml(self):
        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = C.c_void_p()
            ok = False
            if self.pci:
                ok = lib.nvmlDeviceGetHandleByPciBusId_v2(self.pci.encode(), C.byref(h)) == 0
            if not ok:
                ok = lib.nvmlDeviceGetHandleByIndex_v2(self.idx, C.byref(h)) == 0
            if not ok:
                return None
            reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = C.c_uint()
            lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx))  # NVML_CLOCK_SM
            self.max_mhz = float(mx.value)
            return lib, h, reasons
        except (OSError, AttributeError):
            return None

    def _run(self):
        lib, h, reasons = self.nvml
        clk, mask, mw = C.c_uint(), C.c_ulonglong(), C.c_uint()
        while not self._stop.is_set():
            t = time.perf_counter()
            if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and \
                    reasons(h, C.byref(mask)) == 0:
                p = mw.value / 1e3 if lib.nvmlDeviceGetPowerUsage(h, C.byref(mw)) == 0 else None
                self.samples.append((t, float(clk.value), int(mask.value), p))
            self._stop.wait(0.005)

    def start(self):
        import threading
        self.nvml = self._open_nvml()
        if self.nvml is not None:
            self._stop = threading.Event()
            self._thread = threading.Thread(target=self._run, daemon=True)
            self._thread.start()
            time.sleep(0.05)
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None

    def begin(self):
        self.t0 = time.perf_counter()

    def end(self):
        self.t1 = time.perf_counter()

    def stop(self) -> dict:
        if self.nvml is not None:
            self._stop.set()
            self._thread.join()
            lo, hi = self.t0 or 0.0, self.t1 or float("inf")
            inside = [x for x in self.samples if lo <= x[0] <= hi]
            if not inside:
                return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": ["no samples"],
                        "samples": 0, "source": "nvml"}
            masks = 0
            for x in inside:
                masks |= x[2]
            pw = [x[3] for x in inside if x[3] is not None]
            return {"sm_mhz": statistics.median(x[1] for x in inside),
                    "sm_min_mhz": min(x[1] for x in inside), "sm_max_mhz": self.max_mhz,
                    "reasons": sorted(v for k, v in self.REASONS.items() if masks & k),
                    "power_w_median": statistics.median(pw) if pw else None,
                    "samples": len(inside), "source": "nvml, 5 ms, inside the timed region"}
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
                "samples": len(rows), "source": "nvidia-smi, 200 ms"}


def pci_bus_id(torch, dev) -> str | None:
    """The device's PCI address in NVML's form, where torch reports it."""
    p = torch.cuda.get_device_properties(dev)
    try:
        return f"{p.pci_domain_id:08x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
    except AttributeError:
        return None


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
    torch.cuda.empty_cache()
    return n ** 3 / best / 1e12


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "source": "fallback"}


def kernel_roofline(torch, dev, model, box, camera, n, seconds, sgemm_tinst=None) -> dict:
    """Roofline of one fit launch (gaussmle_gb300.roofline): the bound is the
    slowest of the FP32 pipe (FP32 lane operations at 128 per SM per clock),
    the SFU pipe, the FP64 pipe and HBM, each at its peak.  The FP32 peak is
    taken at the GPU's maximum SM clock (MEASURED_PEAKS.json)."""
    from gaussmle_gb300 import roofline
    peaks = measured_peaks()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    mhz = float(peaks.get("sm_max_mhz", 2070.0))
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    r = roofline.roofline(model, box, camera, n, seconds, sms, mhz, hbm)
    out = {"bound": r["bound"], "achieved": r["achieved_tinst"], "peak": r["peak_tinst"],
           "unit": "Tinst/s", "frac": r["frac"], "pipe_frac": r["pipe_frac"],
           "issue_unpacked_frac": r["issue_unpacked_frac"],
           "work_per_roi": r["work"], "bytes_per_roi": r["bytes_per_roi"],
           "hbm": {"achieved_gbs": n * r["bytes_per_roi"] / seconds / 1e9, "peak_gbs": hbm,
                   "frac": r["pipe_frac"]["hbm"]},
           "peak_source": (f"FP32 peak {sms} SMs x 128 lanes x {mhz:.0f} MHz "
                           f"({'MEASURED_PEAKS.json' if 'source' not in peaks else 'fallback'}"
                           " sm_max_mhz); HBM: measured copy bandwidth")}
    if sgemm_tinst is not None:
        out["sgemm_fp32_tinst"] = sgemm_tinst
        out["frac_of_sgemm_rate"] = r["achieved_tinst"] / sgemm_tinst
    return out


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_seed(base: int, rank: int) -> int:
    """Each rank fits its own ROIs (weak scaling: a shard of ROIs per GPU)."""
    return base + rank


def max_over_ranks(x: float, world: int, device="cpu") -> float:
    """The largest x over the job's ranks (one all-reduce; x itself when
    world == 1).  device: where the process group's backend reduces (a CUDA
    device for NCCL, the CPU for gloo)."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: int, steps: int, world: int, seconds_max: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time."""
    return units_per_rank * steps * world / seconds_max


def set_maps(ctx, maps):
    # (ny, nx) column-major maps are stored as row-major (nx, ny) tensors
    v, g, o = (maps[k].cpu().numpy() for k in ("var", "gain", "offset"))
    ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, v.ctypes.data_as(C.c_void_p),
                                           g.ctypes.data_as(C.c_void_p),
                                           o.ctypes.data_as(C.c_void_p), maps["ny"], maps["nx"]))


# ---------------------------------------------------------------------------

def oracle_sample(groups, maps, m_total: int, threads: int):
    """Time the FP32 CPU restatement on a proportional sample of the batch:
    the first m_g ROIs of each group.  run() returns the oracle's outputs."""
    sys.path.insert(0, str(ROOT))
    from oracle import oracle as O
    var, gain, off = (maps[k].cpu().numpy().T for k in ("var", "gain", "offset"))
    n_all = sum(g["n"] for g in groups)
    jobs = []
    for g in groups:
        m = max(1, int(round(m_total * g["n"] / n_all)))
        box = g["box"]
        data = g["data"][: m * box * box].cpu().numpy().reshape(m, box, box).transpose(2, 1, 0)
        c = g["constraints"]
        d = O.make_desc(g["model"], box, 20, g["camera"], g["psf"].psf_vector(), c.lower,
                        c.upper, c.max_step)
        jobs.append((d, data, g["xc"][:m].cpu().numpy(), g["yc"][:m].cpu().numpy(), m))

    def run():
        return [O.fit(d, data, xc, yc, (var, gain, off), "f32", threads)
                for d, data, xc, yc, m in jobs]

    run.jobs = jobs
    run.maps = (var, gain, off)
    return run, sum(j[4] for j in jobs), O.max_threads()


def parity_report(run, outs, gpu_out, groups, n_fp64: int = 3000) -> dict:
    """Parity of the GPU's outputs for the oracle sample's ROIs (the same
    ROIs of the timed batch) against the FP32 oracle, and of both against the
    FP64 oracle on the first n_fp64 ROIs of each group plus every ROI that
    misses the bar (at most 2000 of them per group)."""
    from oracle import oracle as O
    from oracle import parity
    rep = {"bar": "pos/sigma/z 1e-3, N/bg 1e-4 rel, CRLB 1e-3 rel, same flag",
           "reference_bar": "test/gpu_tests.jl:224-226", "groups": []}
    tot = ok = 0
    for (d, data, xc, yc, m), f32, g, go in zip(run.jobs, outs, groups, gpu_out):
        gpu = {k: go[k][:m] for k in ("params", "crlb", "llr", "flags")}
        okm, _ = parity.compare(g["model"], gpu["params"], gpu["crlb"], gpu["flags"], f32)
        miss = np.nonzero(~okm)[0][:2000]
        sel = np.unique(np.concatenate([np.arange(min(m, n_fp64)), miss]))
        sub = data[:, :, sel]
        f64 = O.fit(d, sub, xc[sel], yc[sel], run.maps, "f64")
        gf = O.final_at(d, sub, gpu["params"][sel], xc[sel], yc[sel], run.maps, "f64")
        ff = O.final_at(d, sub, f32["params"][sel], xc[sel], yc[sel], run.maps, "f64")
        st = parity.group_report(g["model"], gpu, f32, f64, sel, gf, ff)
        st.update({"model": g["psf"].__class__.__name__, "box": g["box"]})
        rep["groups"].append(st)
        tot += st["n"]
        ok += st["n"] - st["misses"]
    rep["rois"] = tot
    rep["pass_frac"] = ok / max(tot, 1)
    return rep


def host_cpu() -> str:
    """The host CPU's model and core count (/proc/cpuinfo, else platform)."""
    import platform
    name = None
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read()
        for key in ("model name", "Model Name", "CPU part"):
            for line in info.splitlines():
                if line.startswith(key):
                    name = line.split(":", 1)[1].strip()
                    break
            if name:
                break
        if name and name.lower().startswith("0xd4f"):  # Arm CPU part number
            name = "Arm Neoverse-V2"
    except OSError:
        pass
    return f"{name or platform.processor() or platform.machine()}, {os.cpu_count()} cores"


def cpu_baseline(groups, maps, seconds: float, gpu_out=None) -> dict:
    run, m, nth = oracle_sample(groups, maps, 4000, 0)
    t0 = time.perf_counter()
    run()
    t0 = time.perf_counter() - t0
    scale = max(1.0, seconds / max(t0, 1e-6))
    run, m, nth = oracle_sample(groups, maps, int(4000 * scale), 0)
    t = time.perf_counter()
    outs = run()
    t = time.perf_counter() - t
    out = {"value": m / t, "unit": UNIT, "cores": nth, "kind": "port", "cpu": host_cpu(),
           "sample": f"{m} ROIs of the mixed batch, in its proportions (the first ROIs of each "
                     f"group; {t:.1f} s on {nth} host threads; FP32 restatement of the "
                     "reference CPU path, oracle/gmle_oracle.c)"}
    if gpu_out is not None:
        out["parity"] = parity_report(run, outs, gpu_out, groups)
    return out


def run_reference(args):
    world, rank, local = dist_init()
    if rank != 0:
        return
    import torch
    from gaussmle_gb300 import simulate
    dev = "cuda:0" if torch.cuda.is_available() else "cpu"
    maps, groups = simulate.mixed_batch_scmos_device(n=min(args.n, 200_000), device=dev)
    per_step = 20_000
    run, m, nth = oracle_sample(groups, maps, per_step, 0)
    for _ in range(args.warmup):
        run()
    t = time.perf_counter()
    for _ in range(args.steps):
        run()
    dt = time.perf_counter() - t
    value = m * args.steps / dt
    sample = (f"{m} ROIs of the mixed batch per step on {nth} host threads (FP32 restatement "
              "of the reference CPU path, oracle/gmle_oracle.c; the Julia reference is not "
              "installable here)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rois_per_step": m, "iterations": 20},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                         "cpu": host_cpu(), "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ---------------------------------------------------------------------------

def device_groups(torch, groups, dev):
    from gaussmle_gb300 import serve
    out = []
    for g in groups:
        n, P = g["n"], g["psf"].nparams
        b = {"params": torch.empty((n, P), device=dev), "crlb": torch.empty((n, P), device=dev),
             "llr": torch.empty(n, device=dev), "flags": torch.empty(n, dtype=torch.uint8,
                                                                        device=dev)}
        b["group"] = serve.make_group(g["psf"], g["box"], g["camera"], g["constraints"],
                                      g["data"], g["xc"], g["yc"], b["params"], b["crlb"],
                                      b["llr"], b["flags"])
        out.append(b)
    return out


def time_steps(torch, stream, fn, steps, warmup):
    for _ in range(max(warmup, 3)):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3


def plain_in_fresh_process(model, box, camera, n, steps, method="newton") -> dict:
    """One `--plain` measurement in a process of its own: the launch's time
    does not depend on the workloads this process ran before (in-process, after
    other workloads, the same compute-bound launch was measured up to 9 %
    slower, the full-Hessian one up to 1.8x, with the GPU at full clock)."""
    cmd = [sys.executable, str(ROOT / "bench.py"), "--plain", f"{model},{box},{camera},{n}",
           "--steps", str(steps), "--warmup", "3", "--method", method]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    if res.returncode != 0:
        raise RuntimeError(f"plain run {cmd[3:]} failed:\n{res.stderr[-2000:]}")
    return json.loads(res.stdout.strip().splitlines()[-1])


def extras(torch, ctx, dev, steps, peak_inst):
    """Plain-kernel throughput of the other workloads (device-resident); the
    fit workloads each in a fresh process (plain_in_fresh_process)."""
    out = {}
    for name, model, box, cam, n in [("xynb-11x11-poisson-10k (reference CPU case)", 0, 11, 0, 10_000),
                                     ("xynb-11x11-poisson-1e6", 0, 11, 0, 1_000_000),
                                     ("xynbs-13x13-scmos-1e6", 1, 13, 2, 1_000_000),
                                     ("astig-15x15-poisson-1e6", 3, 15, 0, 1_000_000)]:
        r = plain_in_fresh_process(model, box, cam, n, steps)
        rl = r["roofline"]
        out[name] = {"fits_per_s": r["fits_per_s"], "ms_per_launch": r["ms_per_launch"],
                     "shape": r["shape"], "work_slots_per_roi": rl["work_per_roi"]["slots"],
                     "roofline_frac": rl["frac"], "bound": rl["bound"]}
        if name == "xynb-11x11-poisson-1e6":
            # the full-Hessian option (Fisher scoring with LM damping) on the
            # same ROIs, 20 iterations
            lm = plain_in_fresh_process(model, box, cam, n, steps, "lm")
            out["xynb-11x11-poisson-1e6-fisher-lm"] = {
                "fits_per_s": lm["fits_per_s"], "ms_per_launch": lm["ms_per_launch"],
                "vs_newton": r["ms_per_launch"] / lm["ms_per_launch"]}
    import gaussmle_gb300 as G
    stream = torch.cuda.Stream(dev)
    # ROI extraction from device-resident frames (gmle_cut_rois_device): an
    # HBM-bound copy; 100 frames of 2048 x 2048 (1.7 GB) and 2e6 11x11 ROIs
    # (0.97 GB out), both larger than L2
    box, n, nf = 11, 2_000_000, 100
    gen = torch.Generator(device=dev)
    gen.manual_seed(5)
    frames = torch.rand((nf, 2048, 2048), device=dev, generator=gen)
    ri = lambda hi: torch.randint(1, hi, (n,), device=dev, dtype=torch.int32, generator=gen)
    fidx, xc, yc = ri(nf + 1), ri(2048 - box + 2), ri(2048 - box + 2)
    rois = torch.empty(n * box * box, device=dev)
    dt = time_steps(torch, stream, lambda: G.cut_rois(ctx, frames, fidx, xc, yc, box, out=rois,
                                                      stream=stream), steps, 3)
    per = dt / steps
    peak = measured_peaks().get("hbm_gbs", 6800.0)
    gbs = n * (2 * box * box * 4 + 12) / per / 1e9
    out["roi-cut-11x11-2e6-from-100-frames-2048x2048"] = {
        "rois_per_s": n / per, "ms_per_launch": per * 1e3, "achieved_gbs": gbs,
        "hbm_frac": gbs / peak, "bytes_per_roi": 2 * box * box * 4 + 12}
    # the device ROI generator: 2e6 XYNB 11x11 sCMOS ADU ROIs at random corners
    from gaussmle_gb300.fitter import make_desc
    from gaussmle_gb300.models import GaussianXYNB
    from gaussmle_gb300.constraints import default_constraints
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    u = lambda lo, hi: lo + (hi - lo) * torch.rand(n, generator=g, device=dev)
    truth = torch.stack([u(4.5, 7.5), u(4.5, 7.5), torch.exp(u(np.log(100.0), np.log(20000.0))),
                         u(1, 20)], 1).contiguous()
    psf = GaussianXYNB(1.3)
    desc = make_desc(psf, box, 20, default_constraints(psf, box), 2)
    xc = torch.randint(1, 2048 - box + 2, (n,), generator=g, device=dev, dtype=torch.int32)
    yc = torch.randint(1, 2048 - box + 2, (n,), generator=g, device=dev, dtype=torch.int32)
    rois = torch.empty(n * box * box, device=dev)
    dt = time_steps(torch, stream, lambda: G.simulate_rois(ctx, desc, truth, 5, xc, yc, out=rois,
                                                            stream=stream), steps, 3)
    per = dt / steps
    out["roi-generator-11x11-scmos-adu-2e6"] = {
        "rois_per_s": n / per, "ms_per_launch": per * 1e3,
        "output_gbs": n * box * box * 4 / per / 1e9}
    del frames, rois, fidx, xc, yc, truth
    torch.cuda.empty_cache()
    return out


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
    from gaussmle_gb300 import simulate, roofline, serve, loadgen

    n = args.n
    maps, groups = simulate.mixed_batch_scmos_device(n=n, seed=rank_seed(1003, rank), device=dev)
    ctx = G.Context(local)
    set_maps(ctx, maps)
    dgs = device_groups(torch, groups, dev)
    gstructs = [b["group"] for b in dgs]
    stream = torch.cuda.Stream(dev)
    # launch shapes: the autotuner on each group's data (set-up, not timed)
    from gaussmle_gb300 import tuning
    shapes = []
    for g, b in zip(groups, dgs):
        tpr, rpb, _ = tuning.autotune(ctx, b["group"].desc, g["data"], g["xc"], g["yc"],
                                      b["params"], b["crlb"], b["llr"], b["flags"], save=False)
        shapes.append((tpr, rpb))

    # ---- value: the whole batch through gmle_fit_mixed_device per step ----
    def step():
        serve.fit_mixed_device(ctx, gstructs, stream=stream)

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    launches0 = ctx.launches()
    sampler = ClockSampler(local, pci_bus_id(torch, dev))
    sampler.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("value")  # the timed region, for profiler filters
    sampler.begin()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    sampler.end()
    torch.cuda.nvtx.range_pop()
    clocks = sampler.stop()
    dt = max_over_ranks(e0.elapsed_time(e1) / 1e3, world, dev)
    if world > 1:
        dist.barrier()
    launches = ctx.launches() - launches0
    value = job_rate(n, args.steps, world, dt)
    # the timed step's outputs (host copies, outside the timed region), for
    # the parity check of the oracle sample's ROIs
    gpu_out = [{k: b[k].cpu().numpy() for k in ("params", "crlb", "llr", "flags")} for b in dgs]
    per_step = dt / args.steps
    conv = float(np.mean([(b["flags"].cpu().numpy() & 1).mean() for b in dgs]))

    # ---- each group's launch alone: the dominant kernel and its roofline ----
    per_group = []
    for g, b in zip(groups, dgs):
        fn = (lambda g=g, b=b: G.fit_device(ctx, b["group"].desc, g["data"], g["xc"], g["yc"],
                                             b["params"], b["crlb"], b["llr"], b["flags"],
                                             stream=stream))
        # one range per group (e.g. "group_AstigmaticXYZNB_15"), for profiler filters
        torch.cuda.nvtx.range_push(f"group_{g['psf'].__class__.__name__}_{g['box']}")
        per_group.append(time_steps(torch, stream, fn, args.steps, 3) / args.steps)
        torch.cuda.nvtx.range_pop()
    dt_plain_dev = sum(per_group) * args.steps

    # ---- the same batch as requests of <= 50000 ROIs: table launches only ----
    from gaussmle_gb300 import _lib
    chunks = []
    for g, b in zip(groups, dgs):
        b2, P = g["box"] ** 2, g["psf"].nparams
        for lo in range(0, g["n"], 50_000):
            hi = min(g["n"], lo + 50_000)
            c = _lib.Group()
            c.desc = b["group"].desc
            c.data = C.c_void_p(g["data"].data_ptr() + 4 * lo * b2)
            c.x_corners = C.c_void_p(g["xc"].data_ptr() + 4 * lo)
            c.y_corners = C.c_void_p(g["yc"].data_ptr() + 4 * lo)
            c.n = hi - lo
            c.params = C.c_void_p(b["params"].data_ptr() + 4 * lo * P)
            c.crlb = C.c_void_p(b["crlb"].data_ptr() + 4 * lo * P)
            c.llr = C.c_void_p(b["llr"].data_ptr() + 4 * lo)
            c.flags = C.c_void_p(b["flags"].data_ptr() + lo)
            chunks.append(c)
    l0 = ctx.launches()
    dt_tables = time_steps(torch, stream, lambda: serve.fit_mixed_device(ctx, chunks, stream=stream),
                           args.steps, 3)
    table_only = {"value": n * args.steps / dt_tables, "unit": UNIT, "groups": len(chunks),
                  "launches_per_step": (ctx.launches() - l0) // (args.steps + 3),
                  "api": "gmle_fit_mixed_device, groups of <= 50000 ROIs (device-resident)"}

    # ---- e2e: served requests (pinned host buffers) vs per-request plain calls ----
    e2e, plain, latency = None, None, None
    if not args.no_e2e or not args.no_latency:
        pools = loadgen.HostPools(groups)
        reqs = loadgen.make_stream(pools, n, seed=rank_seed(7, rank))
        srv = serve.Server(ctx, max_inflight_steps=args.max_inflight,
                           use_graphs=bool(args.server_graphs),
                           max_step_rois=args.max_step_rois)
        try:
            if not args.no_e2e:
                # one gmle_submit per request, its descriptor built inside the
                # timed region (requests reach the server one by one and the
                # first steps start while later requests are still submitted)
                for _ in range(max(1, min(args.warmup, 2))):
                    loadgen.run_batch_served(srv, pools, reqs)
                srv.stats(reset=True)
                l0 = ctx.launches()
                if world > 1:
                    dist.barrier()
                ts = [loadgen.run_batch_served(srv, pools, reqs) for _ in range(args.steps)]
                st = srv.stats()
                et = max_over_ranks(sum(ts), world, dev)
                launches_e2e = ctx.launches() - l0
                # the same steps through one gmle_submit_many call per step,
                # with the descriptors built beforehand
                garr = loadgen.group_array(pools, reqs)
                loadgen.run_batch_served(srv, pools, reqs, garr)
                ts1 = [loadgen.run_batch_served(srv, pools, reqs, garr) for _ in range(args.steps)]
                h2d = sum(r.n * (groups[r.group]["box"] ** 2 * 4 + 8) for r in reqs)
                d2h = sum(r.n * (2 * groups[r.group]["psf"].nparams * 4 + 5) for r in reqs)
                e2e = {"value": job_rate(n, args.steps, world, et), "unit": UNIT,
                       "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                       "gpu_launches": launches_e2e, "ms_per_step": et / args.steps * 1e3,
                       "requests_per_step": len(reqs),
                       "api": "gmle_submit per request (descriptor built per request) / gmle_wait",
                       "server_p50_ms": st["p50_latency_ms"], "server_p99_ms": st["p99_latency_ms"],
                       "submit_many": {
                           "value": job_rate(n, args.steps, world,
                                             max_over_ranks(sum(ts1), world, dev)),
                           "unit": UNIT,
                           "api": "one gmle_submit_many per step, descriptors built beforehand"}}
                loadgen.run_batch_plain(ctx, pools, reqs[:50])
                tp = loadgen.run_batch_plain(ctx, pools, reqs)
                plain = {"per_request_gmle_fit": {"value": n / tp, "unit": UNIT,
                                                  "ms_per_step": tp * 1e3,
                                                  "api": "gmle_fit per request"},
                         "one_launch_per_group_device": {"value": n * args.steps / dt_plain_dev,
                                                         "unit": UNIT}}
            if not args.no_latency:
                latency = {"served": [], "plain": [], "served_10k": [], "plain_10k": []}
                for load in [float(x) for x in args.loads.split(",")]:
                    tot = min(args.load_rois, load * 1.5)
                    lreqs = loadgen.make_stream(pools, int(tot), seed=13)
                    latency["served"].append(loadgen.run_stream_served(srv, pools, lreqs, load))
                    latency["plain"].append(loadgen.run_stream_plain(ctx, pools, lreqs, load))
                # requests of exactly 10 000 ROIs (the p99 < 10 ms target's request size)
                for load in [float(x) for x in args.loads_10k.split(",")]:
                    tot = min(args.load_rois, load * 1.5)
                    lreqs = loadgen.make_stream(pools, int(tot), seed=17, lo=10_000, hi=10_000)
                    latency["served_10k"].append(loadgen.run_stream_served(srv, pools, lreqs, load))
                    latency["plain_10k"].append(loadgen.run_stream_plain(ctx, pools, lreqs, load))
        finally:
            srv.stop()

    if rank != 0:
        return
    # ---- roofline of the dominant kernel: FP32, SFU and FP64 pipes and HBM ----
    # (the batch plan gives each group of >= 65536 ROIs its own plain launch)
    k = int(np.argmax(per_group))
    gk = groups[k]
    tpr, rpb = shapes[k]
    peak_inst = fp32_peak_tinst(torch, dev)
    kname = (f"{'fit_kernel_r1' if tpr == 1 else 'fit_kernel'}<{gk['model']}, {gk['box']}, "
             f"{str(gk['camera'] != 0).lower()}, false>")
    traffic = TRAFFIC_BYTES_PER_ROI.get(kname)
    rl = kernel_roofline(torch, dev, gk["model"], gk["box"], gk["camera"], gk["n"],
                         per_group[k], peak_inst)
    rl.update({
        "traffic": traffic * gk["n"] if traffic is not None else None,
        "kernel": f"{kname} (tpr {tpr}, {rpb} ROIs/block), {gk['n']} ROIs per launch",
        "ms_per_launch": per_group[k] * 1e3,
        "launches": [{"model": g["psf"].__class__.__name__, "box": g["box"], "n": g["n"],
                      "shape": list(sh), "ms": t * 1e3,
                      "frac": kernel_roofline(torch, dev, g["model"], g["box"], g["camera"],
                                              g["n"], t)["frac"]}
                     for g, sh, t in zip(groups, shapes, per_group)],
    })
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        cpu = cpu_baseline(groups, maps, args.cpu_seconds, gpu_out)
    ext = None
    if not args.no_extras and world == 1:
        del dgs
        torch.cuda.empty_cache()
        ext = extras(torch, ctx, dev, max(3, args.steps // 2), peak_inst)
    if e2e is not None and plain is not None:
        # the served form against the reference's one-call-per-batch pattern
        # on the same requests
        e2e["served_over_plain"] = e2e["value"] / plain["per_request_gmle_fit"]["value"]
        e2e["plain_per_request_fits_per_s"] = plain["per_request_gmle_fit"]["value"]
    if e2e is not None and latency is not None:
        e2e["latency"] = {
            "served_p99_ms": {f"{x['offered_rois_per_s']:.0e}": x["p99_ms"]
                              for x in latency["served"]},
            "served_p50_ms": {f"{x['offered_rois_per_s']:.0e}": x["p50_ms"]
                              for x in latency["served"]},
            "plain_p99_ms": {f"{x['offered_rois_per_s']:.0e}": x["p99_ms"]
                             for x in latency["plain"]},
            "served_10k_p99_ms": {f"{x['offered_rois_per_s']:.0e}": x["p99_ms"]
                                  for x in latency["served_10k"]},
            "plain_10k_p99_ms": {f"{x['offered_rois_per_s']:.0e}": x["p99_ms"]
                                 for x in latency["plain_10k"]},
            "requests": "log-uniform 50..50000 ROIs (10k: exactly 10 000), Poisson arrivals, "
                        "p50/p99 submit -> results on host"}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "rois_per_step": n,
                   "groups": [{"model": g["psf"].__class__.__name__, "box": g["box"],
                               "n": g["n"]} for g in groups],
                   "parallelism": f"roi-shard x{world}",
                   "l2": "inputs (~1.4 GB/step) larger than L2"},
        "gpu_launches": launches,
        "converged_fraction": conv,
        "clocks": clocks,
        "roofline": rl,
        "e2e": e2e,
        "plain": plain,
        "latency": latency,
        "table_launches": table_only,
        "cpu_baseline": cpu,
        "extras": ext,
    }
    print(json.dumps(out))


def run_plain(args):
    """One homogeneous device-resident workload, plain launches only."""
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    import gaussmle_gb300 as G
    from gaussmle_gb300 import simulate, tuning
    from gaussmle_gb300.fitter import make_desc
    model, box, cam, n = (int(float(x)) for x in args.plain.split(","))
    ctx = G.Context(0)
    wl = simulate.device_workload(model, box, cam, n, device=dev)
    if cam:
        set_maps(ctx, wl)
    psf, P = wl["psf"], wl["psf"].nparams
    cons = simulate.ASTIG_WIDE if model == 3 else G.default_constraints(psf, 11)
    from gaussmle_gb300 import _lib
    method = _lib.METHOD_FISHER_LM if args.method == "lm" else _lib.METHOD_NEWTON
    desc = make_desc(psf, box, 20, cons, cam, method)
    prm = torch.empty((n, P), device=dev)
    crl = torch.empty((n, P), device=dev)
    llr = torch.empty(n, device=dev)
    flg = torch.empty(n, dtype=torch.uint8, device=dev)
    if args.tpr:
        ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, model, box, cam, args.tpr, args.rpb))
        tpr, rpb = args.tpr, args.rpb
    else:
        tpr, rpb, _ = tuning.autotune(ctx, desc, wl["data"], wl["xc"], wl["yc"], prm, crl, llr,
                                      flg, save=False)
    stream = torch.cuda.Stream(dev)
    l0 = ctx.launches()
    dt = time_steps(torch, stream, lambda: G.fit_device(ctx, desc, wl["data"], wl["xc"],
                                                         wl["yc"], prm, crl, llr, flg,
                                                         stream=stream), args.steps,
                    args.warmup)
    per = dt / args.steps
    rl = kernel_roofline(torch, dev, model, box, cam, n, per)
    print(json.dumps({"workload": f"plain model {model} box {box} camera {cam} n {n}"
                                  f" method {args.method}",
                      "fits_per_s": n / per, "ms_per_launch": per * 1e3, "shape": [tpr, rpb],
                      "launches": ctx.launches() - l0, "roofline": rl}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.plain:
        run_plain(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
