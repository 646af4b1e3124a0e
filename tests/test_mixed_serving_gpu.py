"""GPU tests of the mixed-batch persistent kernel and the serving loop.

* The persistent table launches of a heterogeneous batch give the same
  results as the plain kernel on each group alone (same arithmetic and launch
  shape: bit-identical), also for hundreds of small groups in one launch.
* Served requests give the same result alone and in a mix, and match the
  FP32 oracle within the parity bar (tests/parity_cases.py).
* Admission: a request that can never fit the HBM budget is rejected;
  requests beyond the free budget queue and complete.
* gmle_submit_many gives the results of one gmle_submit per request and
  stops at the first request it does not accept.
"""
import ctypes as C

import numpy as np
import pytest

import gaussmle_gb300 as G
from gaussmle_gb300 import _lib, serve
from gaussmle_gb300.fitter import make_desc
from oracle import oracle as O
from parity_cases import compare, make_case, oracle_desc

pytestmark = pytest.mark.gpu

MIX = [("xynb-11", 0, 11, 2, 700), ("xynbs-9", 1, 9, 2, 500), ("xynbsxsy-13", 2, 13, 2, 300),
       ("astig-15", 3, 15, 2, 300), ("xynb-7", 0, 7, 2, 130)]


def _set_maps(ctx, maps):
    var, gain, off = (np.asfortranarray(m) for m in maps)
    ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, var.ctypes.data_as(C.c_void_p),
                                           gain.ctypes.data_as(C.c_void_p),
                                           off.ctypes.data_as(C.c_void_p), var.shape[0],
                                           var.shape[1]))


def _cases():
    """The mix on one shared 256x256 sensor (the maps of the first case)."""
    ws = [make_case(*c, seed=11 + k) for k, c in enumerate(MIX)]
    maps = ws[0].maps
    from gaussmle_gb300 import simulate
    out = []
    for k, w in enumerate(ws):
        rng = np.random.Generator(np.random.Philox(100 + k))
        xc, yc = simulate.random_corners(rng, w.n, w.box, 256, 256)
        data = simulate.scmos_rois(rng, w.psf, w.truth, w.box, maps, xc, yc)
        out.append(simulate.Workload(w.name, w.psf, w.box, 2, w.constraints,
                                     np.asfortranarray(data), xc, yc, w.truth, maps=maps))
    return out


def _dev(torch, w):
    dev = torch.device("cuda", 0)
    P = w.psf.nparams
    t = {
        "data": torch.from_numpy(np.ascontiguousarray(w.data.transpose(2, 1, 0)).reshape(-1)).to(dev),
        "xc": torch.from_numpy(w.x_corners).to(dev), "yc": torch.from_numpy(w.y_corners).to(dev),
        "params": torch.full((w.n, P), float("nan"), device=dev),
        "crlb": torch.full((w.n, P), float("nan"), device=dev),
        "llr": torch.full((w.n,), float("nan"), device=dev),
        "flags": torch.zeros(w.n, dtype=torch.uint8, device=dev),
    }
    return t


# Launch shapes forced per kind so that the table launch and the plain launch
# run the same code: both kernels (one and several threads per ROI) are covered.
SHAPES = [(1, 32), (4, 64), (4, 32), (1, 64), (8, 16)]


def test_mixed_launch_matches_plain_kernel(ctx):
    torch = pytest.importorskip("torch")
    ws = _cases()
    _set_maps(ctx, ws[0].maps)
    bufs = [_dev(torch, w) for w in ws]
    groups = [serve.make_group(w.psf, w.box, 2, w.constraints, b["data"], b["xc"], b["yc"],
                               b["params"], b["crlb"], b["llr"], b["flags"])
              for w, b in zip(ws, bufs)]
    try:
        for w, (tpr, rpb) in zip(ws, SHAPES):
            ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, w.psf.model_id, w.box, 2, tpr, rpb))
        l0 = ctx.launches()
        serve.fit_mixed_device(ctx, groups)
        torch.cuda.synchronize()
        # one persistent table launch per (camera family, model, box) present
        assert ctx.launches() - l0 == len(ws)
        for w, b in zip(ws, bufs):
            ref = _dev(torch, w)
            G.fit_device(ctx, make_desc(w.psf, w.box, 20, w.constraints, 2), ref["data"],
                         ref["xc"], ref["yc"], ref["params"], ref["crlb"], ref["llr"], ref["flags"])
            torch.cuda.synchronize()
            for k in ("params", "crlb", "llr", "flags"):
                a, r = b[k].cpu().numpy(), ref[k].cpu().numpy()
                assert np.array_equal(a, r, equal_nan=True), (w.name, k, np.nanmax(np.abs(a - r)))
    finally:
        for w in ws:
            ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, w.psf.model_id, w.box, 2, 0, 0))


def test_table_launch_takes_many_small_groups(ctx):
    """Hundreds of small groups of one kind share a launch: every ROI is fitted
    once, with the result of the plain kernel on the whole batch."""
    torch = pytest.importorskip("torch")
    w = make_case("xynb-9-poisson", 0, 9, 0, 5000, seed=21)
    dev = torch.device("cuda", 0)
    data = torch.from_numpy(np.ascontiguousarray(w.data.transpose(2, 1, 0)).reshape(-1)).to(dev)
    desc = make_desc(w.psf, 9, 20, w.constraints, 0)
    ref = {"params": torch.empty((5000, 4), device=dev), "crlb": torch.empty((5000, 4), device=dev),
           "llr": torch.empty(5000, device=dev), "flags": torch.empty(5000, dtype=torch.uint8,
                                                                        device=dev)}
    out = {k: torch.full_like(v, float("nan")) if v.dtype != torch.uint8 else torch.zeros_like(v)
           for k, v in ref.items()}
    try:
        ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, 0, 9, 0, 1, 32))
        G.fit_device(ctx, desc, data, None, None, ref["params"], ref["crlb"], ref["llr"],
                     ref["flags"])
        # ragged groups of 1..40 ROIs
        rng = np.random.default_rng(3)
        cuts = np.cumsum(rng.integers(1, 41, 400))
        cuts = np.concatenate([[0], cuts[cuts < 5000], [5000]])
        groups = []
        for lo, hi in zip(cuts[:-1], cuts[1:]):
            groups.append(serve.make_group(
                w.psf, 9, 0, w.constraints, data[lo * 81:hi * 81], None, None,
                out["params"][lo:hi], out["crlb"][lo:hi], out["llr"][lo:hi], out["flags"][lo:hi]))
        l0 = ctx.launches()
        serve.fit_mixed_device(ctx, groups)
        torch.cuda.synchronize()
        assert ctx.launches() - l0 == 1
        for k in ref:
            assert np.array_equal(out[k].cpu().numpy(), ref[k].cpu().numpy(), equal_nan=True), k
    finally:
        ctx.check(ctx.lib.gmle_set_tuning(ctx.handle, 0, 9, 0, 0, 0))


def _host_bufs(w):
    P = w.psf.nparams
    return {"data": np.asfortranarray(w.data, np.float32), "xc": w.x_corners, "yc": w.y_corners,
            "params": np.full((w.n, P), np.nan, np.float32),
            "crlb": np.full((w.n, P), np.nan, np.float32),
            "llr": np.full(w.n, np.nan, np.float32), "flags": np.zeros(w.n, np.uint8)}


def _group(w, b):
    return serve.make_group(w.psf, w.box, 2, w.constraints, b["data"], b["xc"], b["yc"],
                            b["params"], b["crlb"], b["llr"], b["flags"])


@pytest.mark.parametrize("graphs", [True, False], ids=["graph-replays", "block-per-tile"])
def test_served_results_same_alone_and_in_mix(ctx, graphs):
    """Graph replays run persistent table launches; direct launches run one
    block per tile: both give the plain kernel's results."""
    ws = _cases()
    _set_maps(ctx, ws[0].maps)
    srv = serve.Server(ctx, hbm_budget_bytes=256 << 20, max_inflight_steps=2, use_graphs=graphs)
    try:
        # alone: one request at a time
        alone = []
        for w in ws:
            b = _host_bufs(w)
            srv.wait(srv.submit(_group(w, b), keep=b), timeout_s=60)
            alone.append(b)
        # in the mix: all requests submitted at once (several copies of each)
        mixed = []
        tickets = []
        for rep in range(3):
            for w in ws:
                b = _host_bufs(w)
                tickets.append(srv.submit(_group(w, b), keep=b))
                mixed.append(b)
        for t in tickets:
            srv.wait(t, timeout_s=120)
        st = srv.stats()
    finally:
        srv.stop()
    assert st["completed"] == len(ws) * 4 and st["failed"] == 0
    assert st["p99_latency_ms"] >= st["p50_latency_ms"] > 0
    for rep in range(3):
        for k, w in enumerate(ws):
            a, b = alone[k], mixed[rep * len(ws) + k]
            for key in ("params", "crlb", "llr", "flags"):
                assert np.array_equal(a[key], b[key], equal_nan=True), (w.name, key)
    # and the served results meet the parity bar against the FP32 oracle
    for w, b in zip(ws, alone):
        ref = O.fit(oracle_desc(O, w), w.data, w.x_corners, w.y_corners, w.maps, "f32")
        ok, s = compare(w.psf.model_id, b["params"], b["crlb"], b["flags"], ref)
        assert s["pass_frac"] >= (0.97 if w.psf.model_id == 3 else 0.995), (w.name, s)


def test_admission_by_hbm_budget(ctx):
    ws = _cases()
    _set_maps(ctx, ws[0].maps)
    w = ws[0]
    srv = serve.Server(ctx, hbm_budget_bytes=1 << 20, max_inflight_steps=2)
    try:
        big = [_host_bufs(w) for _ in range(6)]   # 700 ROIs of 11x11: ~0.4 MB fits alone
        tickets = [srv.submit(_group(w, b), keep=b) for b in big]
        # six of them exceed the 1 MiB arena together: they queue and all complete
        for t in tickets:
            srv.wait(t, timeout_s=120)
        from gaussmle_gb300 import simulate
        rng = np.random.Generator(np.random.Philox(5))
        n = 4000  # ~2.2 MB: can never fit
        xc, yc = simulate.random_corners(rng, n, 11, 256, 256)
        huge = {"data": np.zeros((11, 11, n), np.float32, order="F"), "xc": xc, "yc": yc,
                "params": np.zeros((n, 4), np.float32), "crlb": np.zeros((n, 4), np.float32),
                "llr": np.zeros(n, np.float32), "flags": np.zeros(n, np.uint8)}
        with pytest.raises(G.GaussMLEError) as ei:
            srv.submit(_group(w, huge), keep=huge)
        assert ei.value.status == 5  # GMLE_ADMISSION_REJECTED
        st = srv.stats()
        assert st["completed"] == 6 and st["rejected"] == 1
        assert st["hbm_peak_bytes"] <= st["hbm_budget_bytes"]
        del big
    finally:
        srv.stop()


@pytest.mark.parametrize("pinned", [False, True], ids=["copied-out", "written-in-place"])
@pytest.mark.parametrize("graphs", [True, False], ids=["graph-replays", "block-per-tile"])
def test_many_requests_from_threads(ctx, graphs, pinned):
    """400 small requests submitted and waited for from four threads at once
    (ctypes releases the GIL, so the library sees concurrent calls): each
    slice's results equal those of the same ROIs served as one request.
    Outputs in pageable memory are copied out; outputs in pinned memory are
    written in place by the kernels, and pinned corners read in place."""
    import threading
    torch = pytest.importorskip("torch")

    def out(shape, dtype, fill):
        if not pinned:
            return np.full(shape, fill, dtype)
        t = torch.empty(shape, dtype=torch.uint8 if dtype == np.uint8 else torch.float32,
                        pin_memory=True)
        t.fill_(fill)
        return t.numpy()  # shares the pinned memory

    ws = _cases()
    _set_maps(ctx, ws[0].maps)
    w = ws[0]
    srv = serve.Server(ctx, hbm_budget_bytes=256 << 20, use_graphs=graphs)
    try:
        whole = _host_bufs(w)
        srv.wait(srv.submit(_group(w, whole), keep=whole), timeout_s=60)
        rng = np.random.default_rng(17)
        slices = []
        for _ in range(400):
            lo = int(rng.integers(0, w.n - 1))
            hi = int(min(w.n, lo + rng.integers(1, 121)))
            slices.append((lo, hi))
        outs = [None] * len(slices)
        errors = []

        def worker(part):
            try:
                tickets = []
                for q in part:
                    lo, hi = slices[q]
                    xc, yc = w.x_corners[lo:hi].copy(), w.y_corners[lo:hi].copy()
                    if pinned:  # corners read in place too
                        xc, yc = (torch.from_numpy(c).pin_memory().numpy() for c in (xc, yc))
                    b = {"data": np.asfortranarray(w.data[:, :, lo:hi]), "xc": xc, "yc": yc,
                         "params": out((hi - lo, w.psf.nparams), np.float32, np.nan),
                         "crlb": out((hi - lo, w.psf.nparams), np.float32, np.nan),
                         "llr": out((hi - lo,), np.float32, np.nan),
                         "flags": out((hi - lo,), np.uint8, 0)}
                    outs[q] = b
                    tickets.append(srv.submit(_group(w, b), keep=b))
                for t in tickets:
                    srv.wait(t, timeout_s=120)
            except Exception as e:  # reported below
                errors.append(e)

        threads = [threading.Thread(target=worker, args=(list(range(k, len(slices), 4)),))
                   for k in range(4)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        assert not errors, errors
        st = srv.stats()
    finally:
        srv.stop()
    assert st["failed"] == 0 and st["completed"] == len(slices) + 1
    for (lo, hi), b in zip(slices, outs):
        for key in ("params", "crlb", "llr", "flags"):
            assert np.array_equal(b[key], whole[key][lo:hi], equal_nan=True), (lo, hi, key)


def test_submit_many_matches_one_at_a_time_and_stops_at_a_bad_request(ctx):
    """gmle_submit_many: the same results as one gmle_submit per request; a
    request with a corner outside the map stops it there (GMLE_INVALID_ARG)
    with the requests before it submitted and served."""
    ws = _cases()
    _set_maps(ctx, ws[0].maps)
    srv = serve.Server(ctx, hbm_budget_bytes=256 << 20)
    try:
        one = []
        for w in ws:
            b = _host_bufs(w)
            srv.wait(srv.submit(_group(w, b), keep=b), timeout_s=60)
            one.append(b)
        bufs = [_host_bufs(w) for w in ws]
        tickets = srv.submit_many([_group(w, b) for w, b in zip(ws, bufs)], keep=bufs)
        assert len(tickets) == len(ws)
        for t in tickets:
            srv.wait(t, timeout_s=120)
        for w, a, b in zip(ws, one, bufs):
            for key in ("params", "crlb", "llr", "flags"):
                assert np.array_equal(a[key], b[key], equal_nan=True), (w.name, key)
        # the second request has one corner past the map's edge
        bufs = [_host_bufs(w) for w in ws[:3]]
        bufs[1]["xc"] = bufs[1]["xc"].copy()
        bufs[1]["xc"][min(5, ws[1].n - 1)] = max(ws[1].maps[0].shape) + 1
        groups = [_group(w, b) for w, b in zip(ws[:3], bufs)]
        arr = (_lib.Group * 3)(*groups)
        tk = (C.c_uint64 * 3)()
        done = C.c_int32(-1)
        st = ctx.lib.gmle_submit_many(ctx.handle, arr, 3, tk, C.byref(done))
        assert st == 1 and done.value == 1  # GMLE_INVALID_ARG at request 1
        assert b"corner outside the calibration map" in ctx.lib.gmle_last_error(ctx.handle)
        assert ctx.lib.gmle_wait(ctx.handle, tk[0], int(60e9)) == 0
        for key in ("params", "crlb", "llr", "flags"):
            assert np.array_equal(bufs[0][key], one[0][key], equal_nan=True), key
    finally:
        srv.stop()
