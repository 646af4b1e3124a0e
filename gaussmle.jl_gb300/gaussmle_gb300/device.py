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


def cut_rois(ctx: _lib.Context, frames, frame_idx, x_corners, y_corners, box: int, out=None,
             stream=None):
    """Cut box x box ROIs out of device-resident frames (gmle_cut_rois_device).

    `frames` is a CUDA float32 tensor holding the Julia (ny, nx, nframes)
    column-major stack, i.e. a contiguous torch tensor of shape
    (nframes, nx, ny); frame indices and corners are 1-based int32 CUDA
    tensors.  Returns (or fills) the ROI-major stack of n*box*box floats that
    fit_device takes."""
    import torch
    if not (frames.is_cuda and frames.is_contiguous() and frames.dim() == 3):
        raise ValueError("frames must be a contiguous (nframes, nx, ny) CUDA tensor")
    nframes, nx, ny = frames.shape
    n = x_corners.shape[0]
    if out is None:
        out = torch.empty(n * box * box, dtype=torch.float32, device=frames.device)
    s = stream if stream is not None else torch.cuda.current_stream(frames.device)
    ptr = lambda t: C.c_void_p(t.data_ptr())
    ctx.check(ctx.lib.gmle_cut_rois_device(ctx.handle, ptr(frames), ny, nx, nframes,
                                           ptr(frame_idx), ptr(x_corners), ptr(y_corners), n,
                                           box, ptr(out), C.c_void_p(s.cuda_stream)))
    return out


def simulate_rois(ctx: _lib.Context, desc, truth, seed: int, x_corners=None, y_corners=None,
                  out=None, stream=None):
    """Synthetic ROIs on the device (gmle_simulate_device).

    `desc` is a fit descriptor (make_desc: model, box, camera, psf in pixel
    units); `truth` a contiguous (n, P) float32 CUDA tensor of true parameters
    in the fitted order; sCMOS cameras use the context's calibration maps at
    the 1-based int32 CUDA corners.  Returns (or fills) the ROI-major stack of
    n*box*box floats that fit_device takes."""
    import torch
    if not (truth.is_cuda and truth.is_contiguous() and truth.dim() == 2):
        raise ValueError("truth must be a contiguous (n, P) CUDA tensor")
    n, box = truth.shape[0], desc.box
    if out is None:
        out = torch.empty(n * box * box, dtype=torch.float32, device=truth.device)
    s = stream if stream is not None else torch.cuda.current_stream(truth.device)
    ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(None)
    ctx.check(ctx.lib.gmle_simulate_device(ctx.handle, C.byref(desc), ptr(truth), ptr(x_corners),
                                           ptr(y_corners), n, C.c_uint64(seed), ptr(out),
                                           C.c_void_p(s.cuda_stream)))
    return out
