"""Request streams for the serving benchmark (the streaming workload).

Request sizes are log-uniform in [50, 50000] ROIs, each request one
(model, box) drawn from the mixed-batch proportions, and its ROIs are slices
of pinned host pools (one per group of a mixed batch).  Arrivals are a
Poisson process at a given offered load in ROIs/s.  Two ways to process a
stream are compared:
  served  gmle_submit into the context's serving loop (continuous batching);
  plain   one worker calling the synchronous per-batch gmle_fit for each
          request in arrival order, as GaussMLE.fit does per batch.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from dataclasses import dataclass

import numpy as np

from . import _lib
from .fitter import make_desc
from .serve import Server


@dataclass
class Request:
    group: int
    lo: int
    n: int
    t_arrive: float = 0.0


class HostPools:
    """Pinned host copies of a mixed batch's groups plus output buffers."""

    def __init__(self, groups: list[dict]):
        import torch
        self.g = groups
        self.h = []
        for gr in groups:
            n, P = gr["n"], gr["psf"].nparams
            self.h.append({
                "data": gr["data"].cpu().pin_memory(), "xc": gr["xc"].cpu().pin_memory(),
                "yc": gr["yc"].cpu().pin_memory(),
                "params": torch.empty((n, P), pin_memory=True),
                "crlb": torch.empty((n, P), pin_memory=True),
                "llr": torch.empty(n, pin_memory=True),
                "flags": torch.empty(n, dtype=torch.uint8, pin_memory=True),
            })
        frac = np.array([gr["n"] for gr in groups], float)
        self.p = frac / frac.sum()
        # per group: its fit descriptor (the same for every request of the
        # group, as a client holds it) and its buffers' base addresses
        self.desc = [make_desc(gr["psf"], gr["box"], 20, gr["constraints"], gr["camera"])
                     for gr in groups]
        self.base = [{k: h[k].data_ptr() for k in h} for h in self.h]

    def group_struct(self, r: Request) -> _lib.Group:
        gr, b = self.g[r.group], self.base[r.group]
        b2, P = gr["box"] * gr["box"], gr["psf"].nparams
        return _lib.Group(self.desc[r.group], b["data"] + 4 * b2 * r.lo, b["xc"] + 4 * r.lo,
                          b["yc"] + 4 * r.lo, r.n, b["params"] + 4 * P * r.lo,
                          b["crlb"] + 4 * P * r.lo, b["llr"] + 4 * r.lo, b["flags"] + r.lo)


def group_array(pools: HostPools, reqs: list[Request]):
    """The requests' descriptors as one ctypes array of Group (for
    Server.submit_many)."""
    return (_lib.Group * len(reqs))(*[pools.group_struct(r) for r in reqs])


def make_stream(pools: HostPools, total_rois: int, seed: int = 7, lo: int = 50,
                hi: int = 50000) -> list[Request]:
    """Requests until total_rois: sizes log-uniform [lo, hi] (all `lo` when
    lo == hi), groups by the mix proportions, ROI slices taken round-robin
    from each group's pool."""
    rng = np.random.default_rng(seed)
    cursor = [0] * len(pools.g)
    out, tot = [], 0
    while tot < total_rois:
        gi = int(rng.choice(len(pools.g), p=pools.p))
        n = lo if lo == hi else int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        cap = pools.g[gi]["n"]
        n = min(n, cap)
        if cursor[gi] + n > cap:
            cursor[gi] = 0
        out.append(Request(gi, cursor[gi], n))
        cursor[gi] += n
        tot += n
    return out


def run_batch_served(srv: Server, pools: HostPools, reqs: list[Request], groups=None) -> float:
    """Submit every request at once, wait for all; returns seconds (Python's
    cyclic collector paused meanwhile).  With `groups` (group_array(reqs),
    descriptors built beforehand, as a client holds them) the requests go in
    one gmle_submit_many call; without, one gmle_submit each."""
    import gc
    gc_was = gc.isenabled()
    gc.disable()
    try:
        t0 = time.perf_counter()
        if groups is not None:
            tickets = srv.submit_many(groups)
        else:
            tickets = [srv.submit(pools.group_struct(r)) for r in reqs]
        for t in tickets:
            srv.wait(t)
        return time.perf_counter() - t0
    finally:
        if gc_was:
            gc.enable()


def run_batch_plain(ctx: _lib.Context, pools: HostPools, reqs: list[Request]) -> float:
    """One synchronous gmle_fit per request, in order; returns seconds."""
    t0 = time.perf_counter()
    for r in reqs:
        G = pools.group_struct(r)
        ctx.check(ctx.lib.gmle_fit(ctx.handle, C.byref(G.desc), G.data, G.x_corners,
                                   G.y_corners, G.n, G.params, G.crlb, G.llr, G.flags))
    return time.perf_counter() - t0


def _arrivals(reqs: list[Request], load: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    mean_n = np.mean([r.n for r in reqs])
    gaps = rng.exponential(mean_n / load, len(reqs))
    return np.cumsum(gaps)


def run_stream_served(srv: Server, pools: HostPools, reqs: list[Request], load: float,
                      seed: int = 11) -> dict:
    """Poisson arrivals at `load` ROIs/s into the serving loop.  The client
    submits from one thread and waits from another, blocking in gmle_wait on
    the tickets in submission order (no polling of the server's lock);
    request descriptors are built before the stream starts and Python's
    cyclic collector is paused during it, so that the client itself does not
    turn arrivals into bursts."""
    import gc
    import queue
    at = _arrivals(reqs, load, seed)
    structs = [pools.group_struct(r) for r in reqs]
    srv.stats(reset=True)
    lat = []
    tickets: queue.SimpleQueue = queue.SimpleQueue()

    def waiter():
        while True:
            item = tickets.get()
            if item is None:
                return
            t, ta = item
            srv.wait(t)
            lat.append(time.perf_counter() - ta)

    gc_was = gc.isenabled()
    gc.disable()
    try:
        th = threading.Thread(target=waiter)
        th.start()
        t0 = time.perf_counter()
        for g, a in zip(structs, at):
            now = time.perf_counter() - t0
            if now < a:
                time.sleep(a - now)
            ta = time.perf_counter()
            tickets.put((srv.submit(g), ta))
        tickets.put(None)
        th.join()
        wall = time.perf_counter() - t0
    finally:
        if gc_was:
            gc.enable()
    st = srv.stats()
    lat_ms = np.array(lat) * 1e3
    # p50/p99: submit -> results on host, timed by the serving loop itself;
    # client_*: the same seen by this Python client (adds polling delay)
    return {"offered_rois_per_s": load, "fits_per_s": sum(r.n for r in reqs) / wall,
            "p50_ms": st["p50_latency_ms"], "p99_ms": st["p99_latency_ms"],
            "client_p50_ms": float(np.percentile(lat_ms, 50)),
            "client_p99_ms": float(np.percentile(lat_ms, 99)),
            "requests": len(reqs), "steps": st["steps"]}


def run_stream_plain(ctx: _lib.Context, pools: HostPools, reqs: list[Request], load: float,
                     seed: int = 11) -> dict:
    """The same arrivals served FIFO by one worker with the per-batch gmle_fit."""
    at = _arrivals(reqs, load, seed)
    lat = []
    t0 = time.perf_counter()
    for r, a in zip(reqs, at):
        now = time.perf_counter() - t0
        if now < a:
            time.sleep(a - now)
        G = pools.group_struct(r)
        ctx.check(ctx.lib.gmle_fit(ctx.handle, C.byref(G.desc), G.data, G.x_corners,
                                   G.y_corners, G.n, G.params, G.crlb, G.llr, G.flags))
        lat.append(time.perf_counter() - t0 - a)
    wall = time.perf_counter() - t0
    lat_ms = np.array(lat) * 1e3
    return {"offered_rois_per_s": load, "fits_per_s": sum(r.n for r in reqs) / wall,
            "p50_ms": float(np.percentile(lat_ms, 50)), "p99_ms": float(np.percentile(lat_ms, 99)),
            "requests": len(reqs)}
