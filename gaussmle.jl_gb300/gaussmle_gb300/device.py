"""Device-resident entry: fit ROIs that already live in HBM (torch tensors).

Mirrors the caller that holds CuArrays and passes device pointers to
gmle_fit_device; the launch is asynchronous on the given CUDA stream.
"""
from __future__ import annotations

import ctypes as C

from . import _lib


def fit_device(ctx: _lib.Context, desc: _lib.FitDesc, data, x_corners, y_corners,
               params, crlb, llr, flags=None, stream=None) -> None:
    """Enqueue a fit of data (n*box*box float32, ROI-major) into the outputs.

    All tensors must be contiguous CUDA tensors on ctx's device; `stream` is a
    torch.cuda.Stream (default: torch's current stream)."""
    import torch
    n = params.shape[0]
    for t in (data, params, crlb, llr):
        if not (t.is_cuda and t.is_contiguous()):
            raise ValueError("fit_device needs contiguous CUDA tensors")
    s = stream if stream is not None else torch.cuda.current_stream(data.device)
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else None
    st = ctx.lib.gmle_fit_device(ctx.handle, C.byref(desc), ptr(data), ptr(x_corners),
                                 ptr(y_corners), n, ptr(params), ptr(crlb), ptr(llr),
                                 ptr(flags), C.c_void_p(s.cuda_stream))
    ctx.check(st)
