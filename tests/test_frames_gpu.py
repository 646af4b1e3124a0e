"""ROI extraction from device-resident frames (gmle_cut_rois_device): the
(box, box, n) stack the reference pipeline builds on the host from an image
stack, corners and frame indices (examples/full_pipeline_boxer.jl:72-103)."""
import ctypes as C

import numpy as np
import pytest

import gaussmle_gb300 as G
from gaussmle_gb300.fitter import make_desc
from gaussmle_gb300 import simulate
from parity_cases import make_case

pytestmark = pytest.mark.gpu


def _host_cut(stack, fidx, xc, yc, box):
    """Julia's stack[y:y+box-1, x:x+box-1, f] for each ROI, as (box, box, n)."""
    out = np.empty((box, box, len(xc)), np.float32, order="F")
    for k, (f, x, y) in enumerate(zip(fidx, xc, yc)):
        out[:, :, k] = stack[y - 1:y - 1 + box, x - 1:x - 1 + box, f - 1]
    return out


def _dev_stack(torch, stack):
    # (ny, nx, nframes) column-major == C-contiguous (nframes, nx, ny)
    return torch.from_numpy(np.ascontiguousarray(stack.transpose(2, 1, 0))).cuda()


@pytest.mark.parametrize("box", [5, 7, 11, 15, 32])
def test_cut_matches_host_slicing(ctx, box):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(box)
    ny, nx, nf, n = 300, 261, 7, 2000
    stack = np.asfortranarray(rng.normal(100, 20, (ny, nx, nf)).astype(np.float32))
    fidx = rng.integers(1, nf + 1, n).astype(np.int32)
    xc = rng.integers(1, nx - box + 2, n).astype(np.int32)
    yc = rng.integers(1, ny - box + 2, n).astype(np.int32)
    xc[:3], yc[:3] = 1, 1                                   # corners of the frame
    xc[3:6], yc[3:6] = nx - box + 1, ny - box + 1
    t = lambda a: torch.from_numpy(a).cuda()
    got = G.cut_rois(ctx, _dev_stack(torch, stack), t(fidx), t(xc), t(yc), box)
    torch.cuda.synchronize()
    want = _host_cut(stack, fidx, xc, yc, box)
    got = got.cpu().numpy().reshape(n, box, box).transpose(2, 1, 0)
    assert np.array_equal(got, want)


def test_rois_outside_the_stack_are_nan_and_counted(ctx):
    torch = pytest.importorskip("torch")
    stack = np.asfortranarray(np.ones((64, 64, 3), np.float32))
    fidx = np.array([1, 4, 2, 0, 3], np.int32)      # frame 4 and 0 do not exist
    xc = np.array([1, 1, 55, 1, 1], np.int32)       # x = 55: 55 + 11 - 1 > 64
    yc = np.array([1, 1, 1, 1, 54], np.int32)       # y = 54 fits exactly
    t = lambda a: torch.from_numpy(a).cuda()
    n0 = C.c_int64()
    ctx.check(ctx.lib.gmle_fit_device_errors(ctx.handle, C.byref(n0)))
    out = G.cut_rois(ctx, _dev_stack(torch, stack), t(fidx), t(xc), t(yc), 11)
    torch.cuda.synchronize()
    rois = out.cpu().numpy().reshape(5, 121)
    assert np.isnan(rois[[1, 2, 3]]).all() and (rois[[0, 4]] == 1).all()
    n1 = C.c_int64()
    ctx.check(ctx.lib.gmle_fit_device_errors(ctx.handle, C.byref(n1)))
    assert n1.value == 3


def test_cut_then_fit_equals_fitting_the_host_stack(ctx):
    """Frames -> device ROIs -> fit gives the fit of the host-cut ROIs."""
    torch = pytest.importorskip("torch")
    w = make_case("xynb-11-poisson", 0, 11, 0, 600, seed=5)
    # place the simulated ROIs in a frame stack at known corners
    ny, nx, nf = 128, 128, 4
    rng = np.random.default_rng(9)
    stack = np.asfortranarray(rng.poisson(5.0, (ny, nx, nf)).astype(np.float32))
    fidx = rng.integers(1, nf + 1, 600).astype(np.int32)
    xc = rng.integers(1, nx - 10, 600).astype(np.int32)
    yc = rng.integers(1, ny - 10, 600).astype(np.int32)
    rois_host = _host_cut(stack, fidx, xc, yc, 11)
    t = lambda a: torch.from_numpy(a).cuda()
    d_rois = G.cut_rois(ctx, _dev_stack(torch, stack), t(fidx), t(xc), t(yc), 11)
    desc = make_desc(w.psf, 11, 20, w.constraints, 0)
    outs = []
    for data in (d_rois, torch.from_numpy(
            np.ascontiguousarray(rois_host.transpose(2, 1, 0)).reshape(-1)).cuda()):
        o = [torch.empty((600, 4), device="cuda"), torch.empty((600, 4), device="cuda"),
             torch.empty(600, device="cuda"), torch.empty(600, dtype=torch.uint8, device="cuda")]
        G.fit_device(ctx, desc, data, None, None, *o)
        torch.cuda.synchronize()
        outs.append([x.cpu().numpy() for x in o])
    for a, b in zip(*outs):
        assert np.array_equal(a, b, equal_nan=True)
