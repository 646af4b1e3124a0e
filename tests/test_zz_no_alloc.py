"""gmle_fit_mixed_device_noalloc: the mixed-batch fit whose scratch is the
library's static device array, called through the C ABI.

It serves callers that cannot allocate device memory: a host whose GPU memory
is held by its own pool allocator (CUDA.jl, PyTorch), or code where a
cudaMalloc, which can synchronise the device, is not allowed.

The GPU test fits one heterogeneous batch, spanning both camera families and
several models and box sizes, with the context entry point gmle_fit_mixed_device.
It then makes two calls in a row of the no-allocation entry point on one
stream, each into fresh NaN-filled outputs.  Both calls must match the
context path within the parity tolerances.  No device memory may be taken
between the two calls.  The argument checks run before any CUDA call, so they
are tested on the CPU too.

This file is collected last on purpose: the entry point must work both in a
fresh process and after every other test has used the context paths.
"""
import ctypes as C

import numpy as np
import pytest

from gaussmle_gb300 import _lib, build, serve, simulate
from parity_cases import compare, make_case

MIX = [  # name, model, box, camera, n
    ("xynb-11-poisson", 0, 11, 0, 900), ("astig-15-poisson", 3, 15, 0, 300),
    ("xynbs-7-poisson", 1, 7, 0, 500), ("xynbs-9-adu", 1, 9, 2, 400),
    ("xynbsxsy-13-adu", 2, 13, 2, 300), ("xynb-11-adu", 0, 11, 2, 700),
    ("xynb-5-poisson-empty", 0, 5, 0, 0),
]
SENSOR = 256


def _lib_loaded():
    build.build()
    return _lib.load()


def _workloads():
    """The mix; sCMOS groups share one sensor's calibration maps."""
    maps = simulate.scmos_maps(np.random.Generator(np.random.Philox(77)), SENSOR, SENSOR)
    out = []
    for k, (name, model, box, cam, n) in enumerate(MIX):
        w = make_case(name, model, box, 0, max(n, 1), seed=300 + k)
        if cam:
            rng = np.random.Generator(np.random.Philox(400 + k))
            xc, yc = simulate.random_corners(rng, n, box, SENSOR, SENSOR)
            data = simulate.scmos_rois(rng, w.psf, w.truth[:n], box, maps, xc, yc)
            w = simulate.Workload(name, w.psf, box, cam, w.constraints, np.asfortranarray(data),
                                  xc, yc, w.truth[:n], maps=maps)
        elif n == 0:
            w = simulate.Workload(name, w.psf, box, 0, w.constraints,
                                  np.zeros((box, box, 0), np.float32, order="F"),
                                  w.x_corners[:0], w.y_corners[:0], w.truth[:0])
        out.append(w)
    return out, maps


def _device_buffers(torch, ws):
    dev = torch.device("cuda", 0)
    bufs = []
    for w in ws:
        P, n = w.psf.nparams, w.data.shape[2]
        bufs.append({
            "data": torch.from_numpy(np.ascontiguousarray(w.data.transpose(2, 1, 0)).reshape(-1))
                         .to(dev),
            "xc": torch.from_numpy(np.ascontiguousarray(w.x_corners)).to(dev),
            "yc": torch.from_numpy(np.ascontiguousarray(w.y_corners)).to(dev),
        })
    return bufs


def _outputs(torch, ws):
    dev = torch.device("cuda", 0)
    return [{"params": torch.full((w.data.shape[2], w.psf.nparams), float("nan"), device=dev),
             "crlb": torch.full((w.data.shape[2], w.psf.nparams), float("nan"), device=dev),
             "llr": torch.full((w.data.shape[2],), float("nan"), device=dev),
             "flags": torch.zeros(w.data.shape[2], dtype=torch.uint8, device=dev)} for w in ws]


def _groups(ws, ins, outs):
    gs = [serve.make_group(w.psf, w.box, w.camera, w.constraints, i["data"], i["xc"], i["yc"],
                           o["params"], o["crlb"], o["llr"], o["flags"])
          for w, i, o in zip(ws, ins, outs)]
    return (_lib.Group * len(gs))(*gs)


def test_more_groups_than_the_static_table_are_rejected():
    lib = _lib_loaded()
    groups = (_lib.Group * 1025)()
    err = C.create_string_buffer(256)
    st = lib.gmle_fit_mixed_device_noalloc(groups, 1025, None, None, None, 0, 0, None, err, 256)
    assert st == 1  # GMLE_INVALID_ARG, before any CUDA call
    assert b"1025" in err.value and b"1024" in err.value


def test_invalid_groups_are_rejected_with_a_message():
    lib = _lib_loaded()
    ws, _ = _workloads()
    g = serve.make_group(ws[5].psf, 11, 2, ws[5].constraints, np.zeros(121, np.float32),
                         np.ones(1, np.int32), np.ones(1, np.int32), np.zeros((1, 4), np.float32),
                         np.zeros((1, 4), np.float32), np.zeros(1, np.float32))
    err = C.create_string_buffer(256)
    st = lib.gmle_fit_mixed_device_noalloc(C.byref(g), 1, None, None, None, 0, 0, None, err, 256)
    assert st == 1 and b"variance" in err.value  # an sCMOS group with no maps
    g.desc.box = 17  # boxes above 16 run through gmle_fit / gmle_fit_device only
    st = lib.gmle_fit_mixed_device_noalloc(C.byref(g), 1, None, None, None, 0, 0, None, err, 256)
    assert st == 3 and b"3..16" in err.value  # GMLE_UNSUPPORTED_BOX


@pytest.mark.gpu
def test_noalloc_matches_the_context_entry_point_on_two_calls(ctx):
    torch = pytest.importorskip("torch")
    lib = _lib_loaded()
    ws, maps = _workloads()
    var, gain, off = (np.asfortranarray(m, np.float32) for m in maps)
    ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, var.ctypes.data_as(C.c_void_p),
                                           gain.ctypes.data_as(C.c_void_p),
                                           off.ctypes.data_as(C.c_void_p), SENSOR, SENSOR))
    ins = _device_buffers(torch, ws)
    ref = _outputs(torch, ws)
    stream = torch.cuda.Stream()
    ctx.check(ctx.lib.gmle_fit_mixed_device(ctx.handle, _groups(ws, ins, ref), len(ws),
                                            C.c_void_p(stream.cuda_stream)))
    stream.synchronize()

    # (ny, nx) column-major maps on the device: torch (nx, ny) row-major
    dev = torch.device("cuda", 0)
    d_maps = [torch.from_numpy(np.ascontiguousarray(m.T)).to(dev) for m in (var, gain, off)]
    outs = [_outputs(torch, ws), _outputs(torch, ws)]
    tables = [_groups(ws, ins, o) for o in outs]
    torch.cuda.synchronize()
    free = []
    for call in range(2):
        err = C.create_string_buffer(512)
        st = lib.gmle_fit_mixed_device_noalloc(
            tables[call], len(ws), *(C.c_void_p(m.data_ptr()) for m in d_maps), SENSOR, SENSOR,
            C.c_void_p(stream.cuda_stream), err, 512)
        assert st == 0, err.value
        stream.synchronize()
        free.append(torch.cuda.mem_get_info(0)[0])
    assert free[0] == free[1]  # the second call took no device memory

    for call in range(2):
        for w, r, o in zip(ws, ref, outs[call]):
            if w.data.shape[2] == 0:
                continue
            got = {k: v.cpu().numpy() for k, v in o.items()}
            want = {k: v.cpu().numpy() for k, v in r.items()}
            ok, s = compare(w.psf.model_id, got["params"], got["crlb"], got["flags"], want)
            assert s["pass_frac"] == 1.0, (call, w.name, s)
            assert np.array_equal(got["flags"], want["flags"]), (call, w.name)
            np.testing.assert_allclose(got["llr"], want["llr"], rtol=1e-4, atol=1e-3,
                                       err_msg=f"call {call} {w.name}")


@pytest.mark.gpu
def test_noalloc_many_small_groups_of_two_kinds(ctx):
    """1024 groups (the static table's limit) of 1..300 ROIs of two kinds, most
    of them not a whole number of blocks: each group's tile lookup (a binary
    search over the groups' first tiles) and the arguments at the end of the
    static table, against gmle_fit_mixed_device group by group."""
    torch = pytest.importorskip("torch")
    lib = _lib_loaded()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(11)
    maps = simulate.scmos_maps(np.random.Generator(np.random.Philox(78)), SENSOR, SENSOR)
    var, gain, off = (np.asfortranarray(m, np.float32) for m in maps)
    ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, var.ctypes.data_as(C.c_void_p),
                                           gain.ctypes.data_as(C.c_void_p),
                                           off.ctypes.data_as(C.c_void_p), SENSOR, SENSOR))
    sizes = rng.integers(1, 301, 1024)
    kinds = rng.integers(0, 2, 1024)  # 0: XYNB 11x11 Poisson, 1: XYNBS 9x9 sCMOS ADU
    base = []
    for kind in (0, 1):
        n = int(sizes[kinds == kind].sum())
        w = make_case("xynb-11-poisson", 0, 11, 0, n, seed=500) if kind == 0 else None
        if kind == 1:
            w0 = make_case("xynbs-9-poisson", 1, 9, 0, n, seed=501)
            r = np.random.Generator(np.random.Philox(502))
            xc, yc = simulate.random_corners(r, n, 9, SENSOR, SENSOR)
            data = simulate.scmos_rois(r, w0.psf, w0.truth, 9, maps, xc, yc)
            w = simulate.Workload("xynbs-9-adu", w0.psf, 9, 2, w0.constraints,
                                  np.asfortranarray(data), xc, yc, w0.truth, maps=maps)
        base.append((w, _device_buffers(torch, [w])[0]))
    P = [4, 5]
    outs = [[{"params": torch.full((int(sizes[kinds == k].sum()), P[k]), float("nan"), device=dev),
              "crlb": torch.full((int(sizes[kinds == k].sum()), P[k]), float("nan"), device=dev),
              "llr": torch.full((int(sizes[kinds == k].sum()),), float("nan"), device=dev),
              "flags": torch.zeros(int(sizes[kinds == k].sum()), dtype=torch.uint8, device=dev)}
             for k in (0, 1)] for _ in range(2)]

    def table(o):
        gs, lo = [], [0, 0]
        for n, k in zip(sizes, kinds):
            w, i = base[k]
            a, b2 = lo[k], w.box * w.box
            g = serve.make_group(w.psf, w.box, w.camera, w.constraints, i["data"], i["xc"],
                                 i["yc"], o[k]["params"], o[k]["crlb"], o[k]["llr"],
                                 o[k]["flags"])
            g.data = C.c_void_p(i["data"].data_ptr() + 4 * a * b2)
            g.x_corners = C.c_void_p(i["xc"].data_ptr() + 4 * a)
            g.y_corners = C.c_void_p(i["yc"].data_ptr() + 4 * a)
            g.n = int(n)
            g.params = C.c_void_p(o[k]["params"].data_ptr() + 4 * a * P[k])
            g.crlb = C.c_void_p(o[k]["crlb"].data_ptr() + 4 * a * P[k])
            g.llr = C.c_void_p(o[k]["llr"].data_ptr() + 4 * a)
            g.flags = C.c_void_p(o[k]["flags"].data_ptr() + a)
            gs.append(g)
            lo[k] += int(n)
        return (_lib.Group * len(gs))(*gs)

    stream = torch.cuda.Stream()
    ctx.check(ctx.lib.gmle_fit_mixed_device(ctx.handle, table(outs[0]), 1024,
                                            C.c_void_p(stream.cuda_stream)))
    d_maps = [torch.from_numpy(np.ascontiguousarray(m.T)).to(dev) for m in (var, gain, off)]
    err = C.create_string_buffer(512)
    st = lib.gmle_fit_mixed_device_noalloc(table(outs[1]), 1024,
                                           *(C.c_void_p(m.data_ptr()) for m in d_maps),
                                           SENSOR, SENSOR, C.c_void_p(stream.cuda_stream), err, 512)
    assert st == 0, err.value
    stream.synchronize()
    for k in (0, 1):
        w = base[k][0]
        got = {key: v.cpu().numpy() for key, v in outs[1][k].items()}
        want = {key: v.cpu().numpy() for key, v in outs[0][k].items()}
        assert not np.isnan(got["params"]).any(), f"kind {k}: ROIs left unfitted"
        ok, s = compare(w.psf.model_id, got["params"], got["crlb"], got["flags"], want)
        assert s["pass_frac"] == 1.0, (k, s)
        assert np.array_equal(got["flags"], want["flags"]), k
