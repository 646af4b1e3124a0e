"""Edge cases of the CUDA path and its C ABI: empty and ragged batches, the
initial estimate, invalid corners, unsupported shapes, dark and saturated ROIs,
pinned vs pageable buffers, golden fixtures, the autotuner."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import gaussmle_gb300 as G
from gaussmle_gb300.fitter import make_desc
from oracle import oracle as O
from parity_cases import compare, make_case, oracle_desc

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def host_fit(ctx, desc, data, xc=None, yc=None, n=None):
    n = data.shape[2] if n is None else n
    P = {0: 4, 1: 5, 2: 6, 3: 5}.get(desc.model, 6)
    out = (np.empty((n, P), np.float32), np.empty((n, P), np.float32), np.empty(n, np.float32),
           np.empty(n, np.uint8))
    st = ctx.lib.gmle_fit(ctx.handle, C.byref(desc), p(np.asfortranarray(data, np.float32)),
                          p(xc), p(yc), n, *(p(o) for o in out))
    return st, out


def set_maps(ctx, maps):
    var, gain, off = (np.asfortranarray(m, np.float32) for m in maps)
    ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, p(var), p(gain), p(off), var.shape[0],
                                           var.shape[1]))


@pytest.mark.parametrize("path", sorted(GOLDEN.glob("oracle_*.npz")), ids=lambda q: q.stem)
def test_golden_fixtures(ctx, path):
    g = np.load(path)
    cam = int(g["camera"])
    if cam:
        set_maps(ctx, (g["var"], g["gain"], g["offset"]))
    d = G.FitDesc()
    d.model, d.box, d.iterations, d.camera = int(g["model"]), int(g["box"]), 20, cam
    for t in range(8):
        d.psf[t] = float(g["psf"][t])
    for k in range(len(g["lower"])):
        d.lower[k], d.upper[k], d.max_step[k] = (float(g["lower"][k]), float(g["upper"][k]),
                                                 float(g["max_step"][k]))
    st, (prm, crlb, llr, fl) = host_fit(ctx, d, g["data"], g["xc"], g["yc"])
    ctx.check(st)
    ok, s = compare(int(g["model"]), prm, crlb, fl, {"params": g["params"], "crlb": g["crlb"],
                                                      "flags": g["flags"]})
    assert s["pass_frac"] >= (0.95 if int(g["model"]) == 3 else 1.0), s


def test_empty_batch_is_a_no_op(ctx):
    w = make_case("xynb-11-poisson", 0, 11, 0, 4)
    desc = make_desc(w.psf, 11, 20, w.constraints, 0)
    st, _ = host_fit(ctx, desc, w.data, n=0)
    assert st == 0
    with pytest.raises(ValueError):
        G.fit(G.GaussMLEFitter(), np.zeros((11, 11, 0), np.float32))


def test_zero_iterations_gives_the_reference_initial_estimate(ctx):
    for case in [("xynb-11-poisson", 0, 11, 0, 300), ("astig-15-poisson", 3, 15, 0, 300),
                 ("xynbs-13-scmos-adu", 1, 13, 2, 300)]:
        w = make_case(*case)
        if w.camera:
            set_maps(ctx, w.maps)
        desc = make_desc(w.psf, w.box, 0, w.constraints, w.camera)
        st, (prm, crlb, llr, fl) = host_fit(ctx, desc, w.data, w.x_corners, w.y_corners)
        ctx.check(st)
        ref = O.fit(oracle_desc(O, w, iterations=0), w.data, w.x_corners, w.y_corners, w.maps)
        # same operations in the same order without FMA: bit-identical start point
        assert np.array_equal(prm, ref["params"]), case[0]


def test_ragged_batch_sizes(ctx):
    w = make_case("xynbsxsy-13-scmos-adu", 2, 13, 2, 1000)
    set_maps(ctx, w.maps)
    ref = O.fit(oracle_desc(O, w), w.data, w.x_corners, w.y_corners, w.maps)
    for n in (1, 31, 33, 257, 999):
        desc = make_desc(w.psf, 13, 20, w.constraints, 2)
        st, (prm, crlb, llr, fl) = host_fit(ctx, desc, w.data[:, :, :n], w.x_corners[:n],
                                            w.y_corners[:n])
        ctx.check(st)
        sub = {k: v[:n] for k, v in ref.items()}
        ok, s = compare(2, prm, crlb, fl, sub)
        assert s["pass_frac"] == 1.0, (n, s)


def test_corners_outside_the_map_are_rejected(ctx):
    w = make_case("xynb-15-scmos-adu", 0, 15, 2, 20)
    set_maps(ctx, w.maps)
    desc = make_desc(w.psf, 15, 20, w.constraints, 2)
    xc = w.x_corners.copy()
    xc[7] = 256 - 15 + 2          # one column past the 256-wide map
    st, _ = host_fit(ctx, desc, w.data, xc, w.y_corners)
    assert st == 1  # GMLE_INVALID_ARG
    assert b"outside" in ctx.lib.gmle_last_error(ctx.handle)
    # device entry: the ROI is skipped (NaN, flag 0) and counted
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    data = torch.from_numpy(np.ascontiguousarray(w.data.transpose(2, 1, 0)).reshape(-1)).to(dev)
    out = [torch.empty((20, 4), device=dev), torch.empty((20, 4), device=dev),
           torch.empty(20, device=dev), torch.empty(20, dtype=torch.uint8, device=dev)]
    n0 = C.c_int64()
    ctx.check(ctx.lib.gmle_fit_device_errors(ctx.handle, C.byref(n0)))
    G.fit_device(ctx, desc, data, torch.from_numpy(xc).to(dev),
                 torch.from_numpy(w.y_corners).to(dev), *out)
    n1 = C.c_int64()
    ctx.check(ctx.lib.gmle_fit_device_errors(ctx.handle, C.byref(n1)))
    assert n1.value == 1
    prm = out[0].cpu().numpy()
    assert np.isnan(prm[7]).all() and np.isfinite(np.delete(prm, 7, 0)).all()
    assert out[3].cpu().numpy()[7] == 0


def test_unsupported_shapes_and_models(ctx):
    w = make_case("xynb-11-poisson", 0, 11, 0, 4)
    desc = make_desc(w.psf, 11, 20, w.constraints, 0)
    desc.box = 65  # boxes 3..64 are fitted
    st, _ = host_fit(ctx, desc, np.zeros((65, 65, 4), np.float32))
    assert st == 3  # GMLE_UNSUPPORTED_BOX
    desc.box, desc.model = 11, 9
    st, _ = host_fit(ctx, desc, w.data)
    assert st == 2  # GMLE_UNSUPPORTED_MODEL
    desc.model, desc.camera = 0, 7
    st, _ = host_fit(ctx, desc, w.data)
    assert st == 1


def test_dark_and_saturated_rois_match_oracle(ctx):
    w = make_case("xynb-11-poisson", 0, 11, 0, 64)
    data = np.asfortranarray(w.data.copy())
    data[:, :, :16] = 0.0                    # dark: every pixel zero
    data[:, :, 16:32] *= 1e3                 # very bright
    data[:, :, 32:40] = 5.0                  # flat background, no spot
    desc = make_desc(w.psf, 11, 20, w.constraints, 0)
    st, (prm, crlb, llr, fl) = host_fit(ctx, desc, data)
    ctx.check(st)
    ref = O.fit(oracle_desc(O, w), data)
    ok, s = compare(0, prm, crlb, fl, ref)
    assert s["flag_mismatch"] == 0
    assert ok[16:32].all() and ok[40:].all(), s
    # dark / flat ROIs: both hit the same constraint bounds
    np.testing.assert_allclose(prm[:16], ref["params"][:16], rtol=1e-4, atol=1e-3)


def test_pinned_and_pageable_buffers_agree(ctx):
    torch = pytest.importorskip("torch")
    w = make_case("xynbs-13-scmos-adu", 1, 13, 2, 3000)
    set_maps(ctx, w.maps)
    desc = make_desc(w.psf, 13, 20, w.constraints, 2)
    st, a = host_fit(ctx, desc, w.data, w.x_corners, w.y_corners)
    ctx.check(st)
    hd = torch.from_numpy(np.ascontiguousarray(w.data.transpose(2, 1, 0)).reshape(-1)).pin_memory()
    outs = [torch.empty((3000, 5), pin_memory=True), torch.empty((3000, 5), pin_memory=True),
            torch.empty(3000, pin_memory=True), torch.empty(3000, dtype=torch.uint8,
                                                            pin_memory=True)]
    vp = lambda t: C.c_void_p(t.data_ptr())
    xc = torch.from_numpy(w.x_corners).pin_memory()
    yc = torch.from_numpy(w.y_corners).pin_memory()
    ctx.check(ctx.lib.gmle_fit(ctx.handle, C.byref(desc), vp(hd), vp(xc), vp(yc), 3000,
                               *(vp(o) for o in outs)))
    for x, y in zip(a, outs):
        assert np.array_equal(x, y.numpy())


def test_autotune_picks_a_valid_shape(ctx):
    torch = pytest.importorskip("torch")
    from gaussmle_gb300 import tuning
    w = make_case("xynb-11-poisson", 0, 11, 0, 4000)
    dev = torch.device("cuda", 0)
    data = torch.from_numpy(np.ascontiguousarray(w.data.transpose(2, 1, 0)).reshape(-1)).to(dev)
    out = [torch.empty((4000, 4), device=dev), torch.empty((4000, 4), device=dev),
           torch.empty(4000, device=dev), torch.empty(4000, dtype=torch.uint8, device=dev)]
    desc = make_desc(w.psf, 11, 20, w.constraints, 0)
    try:
        tpr, rpb, ms = tuning.autotune(ctx, desc, data, None, None, *out, save=False)
        assert tpr in (1, 2, 4, 8) and (tpr * rpb) % 32 == 0 and ms > 0
        G.fit_device(ctx, desc, data, None, None, *out)
        torch.cuda.synchronize()
        ref = O.fit(oracle_desc(O, w), w.data)
        ok, s = compare(0, out[0].cpu().numpy(), out[1].cpu().numpy(), out[3].cpu().numpy(), ref)
        assert s["pass_frac"] == 1.0, s
    finally:
        ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, 0, 11, 0, 0, 0))
