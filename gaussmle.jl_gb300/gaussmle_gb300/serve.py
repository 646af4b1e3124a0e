"""Mixed batches and the serving loop from Python (over the C ABI).

fit_mixed_device: groups of device-resident ROIs of any (model, box), one
table launch per kind present (gmle_fit_mixed_device).
Server: the context's request loop (gmle_server_start / gmle_submit /
gmle_wait): admission by HBM budget, continuous batching of requests into
steps of one-block-per-tile table launches (or, with use_graphs, replays of
CUDA graphs of persistent launches), results written in place into pinned
host outputs and pinned corner arrays read in place, p50/p99 latency.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .constraints import ParameterConstraints
from .fitter import make_desc
from .models import PSFModel


def _vp(x):
    if x is None:
        return None
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    return x.ctypes.data_as(C.c_void_p)


def make_group(psf_pixels: PSFModel, box: int, camera: int, constraints: ParameterConstraints,
               data, x_corners, y_corners, params, crlb, llr, flags=None,
               iterations: int = 20) -> _lib.Group:
    """A gmle_group over host (numpy) or device (torch) buffers."""
    g = _lib.Group()
    g.desc = make_desc(psf_pixels, box, iterations, constraints, camera)
    g.data = _vp(data)
    g.x_corners = _vp(x_corners)
    g.y_corners = _vp(y_corners)
    g.n = params.shape[0]
    g.params, g.crlb, g.llr, g.flags = _vp(params), _vp(crlb), _vp(llr), _vp(flags)
    return g


def fit_mixed_device(ctx: _lib.Context, groups: list[_lib.Group], stream=None) -> None:
    """Fit device-resident groups: one persistent table launch per (camera family,
    model, box) present, plain launches for groups of 65536 ROIs or more
    (gmle_fit_mixed_device; the reference's Newton method only)."""
    import torch
    arr = (_lib.Group * len(groups))(*groups)
    s = stream if stream is not None else torch.cuda.current_stream()
    ctx.check(ctx.lib.gmle_fit_mixed_device(ctx.handle, arr, len(groups),
                                            C.c_void_p(s.cuda_stream)))


class Server:
    """The context's serving loop.  Host buffers passed to submit() must stay
    alive until the request is waited for."""

    def __init__(self, ctx: _lib.Context, hbm_budget_bytes: int = 0, max_inflight_steps: int = 0,
                 max_step_rois: int = 0, max_pending: int = 0, use_graphs: bool = False):
        self.ctx = ctx
        cfg = _lib.ServerConfig(hbm_budget_bytes, max_inflight_steps, max_step_rois,
                                max_pending, int(use_graphs))
        ctx.check(ctx.lib.gmle_server_start(ctx.handle, C.byref(cfg)))
        self._keep: dict[int, tuple] = {}

    def submit(self, group: _lib.Group, keep=()) -> int:
        t = C.c_uint64()
        self.ctx.check(self.ctx.lib.gmle_submit(self.ctx.handle, C.byref(group), C.byref(t)))
        self._keep[t.value] = (group, keep)
        return t.value

    def submit_many(self, groups, keep=()) -> list[int]:
        """Submit requests in one call (gmle_submit_many): `groups` is a ctypes
        array of Group (or a list, copied into one).  Returns their tickets;
        raises on the first request not accepted (the ones before it stay
        submitted and their tickets are kept for wait())."""
        n = len(groups)
        arr = groups if isinstance(groups, C.Array) else (_lib.Group * n)(*groups)
        tk = (C.c_uint64 * n)()
        done = C.c_int32()
        st = self.ctx.lib.gmle_submit_many(self.ctx.handle, arr, n, tk, C.byref(done))
        out = list(tk[: done.value])
        for k, t in enumerate(out):
            self._keep[t] = (arr, keep)
        self.ctx.check(st)
        return out

    def wait(self, ticket: int, timeout_s: float | None = None) -> None:
        ns = -1 if timeout_s is None else int(timeout_s * 1e9)
        st = self.ctx.lib.gmle_wait(self.ctx.handle, ticket, ns)
        if st != 7:  # anything but GMLE_TIMEOUT ends the request
            self._keep.pop(ticket, None)
        self.ctx.check(st)

    def poll(self, ticket: int) -> bool:
        st = self.ctx.lib.gmle_poll(self.ctx.handle, ticket)
        if st == 9:  # GMLE_NOT_READY
            return False
        self._keep.pop(ticket, None)
        self.ctx.check(st)
        return True

    def stats(self, reset: bool = False) -> dict:
        s = _lib.ServerStats()
        self.ctx.check(self.ctx.lib.gmle_server_stats_get(self.ctx.handle, C.byref(s), int(reset)))
        return s.as_dict()

    def stop(self) -> None:
        self.ctx.check(self.ctx.lib.gmle_server_stop(self.ctx.handle))
        self._keep.clear()
