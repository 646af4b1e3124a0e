"""CPU tests of the host-side mirror of the reference API (no GPU needed)."""
import ctypes as C
import json

import numpy as np
import pytest

import gaussmle_gb300 as G
from gaussmle_gb300 import _lib, loadgen, roofline, simulate
from gaussmle_gb300.fitter import make_desc, validate_fit_input


def test_default_constraints_match_reference():
    # src/constraints.jl:16-47, built for box 11 by the fitter (src/interface.jl:141)
    c = G.default_constraints(G.GaussianXYNB(0.13), 11)
    assert list(c.lower) == [-2, -2, 1, np.float32(0.01)]
    assert list(c.upper[:2]) == [13, 13] and np.isinf(c.upper[2:]).all()
    assert list(c.max_step) == [1, 1, 100, 2]
    c = G.default_constraints(G.GaussianXYNBS(), 11)
    assert c.lower[4] == np.float32(0.3) and c.upper[4] == 5 and c.max_step[4] == 0.5
    c = G.default_constraints(G.GaussianXYNBSXSY(), 11)
    assert len(c.lower) == 6
    c = G.default_constraints(G.AstigmaticXYZNB(), 11)
    assert (c.lower[2], c.upper[2], c.max_step[2]) == (-1, 1, np.float32(0.1))
    assert G.GaussMLEFitter().constraints.upper[0] == 13


def test_to_pixel_units_matches_reference():
    # src/psf_models.jl:311-331: widths / pixel size; gamma, d unchanged
    assert G.GaussianXYNB(0.13).to_pixel_units(0.1).sigma == pytest.approx(1.3, rel=1e-6)
    a = G.AstigmaticXYZNB(0.13, 0.14, 0.05, 0.06, 0.3, 0.2, 0.05, 0.4).to_pixel_units(0.1)
    assert (a.sx0, a.sy0) == pytest.approx((1.3, 1.4), rel=1e-6)
    assert (a.gamma, a.d, a.Ax, a.By) == (0.05, 0.4, 0.05, 0.2)


def test_validate_fit_input_errors_like_reference():
    # src/interface.jl:10-40
    with pytest.raises(ValueError, match="empty"):
        validate_fit_input(np.zeros((7, 7, 0), np.float32))
    with pytest.raises(ValueError, match="square"):
        validate_fit_input(np.zeros((7, 5, 2), np.float32))
    with pytest.raises(ValueError, match="3x3"):
        validate_fit_input(np.zeros((2, 2, 2), np.float32))
    bad = np.ones((7, 7, 2), np.float32)
    bad[3, 3, 1] = np.nan
    with pytest.raises(ValueError, match="NaN or Inf"):
        validate_fit_input(bad)


def test_fit_desc_carries_model_constants_and_constraints():
    psf = G.AstigmaticXYZNB(1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50.0, 100.0)
    d = make_desc(psf, 15, 20, simulate.ASTIG_WIDE, 2)
    assert (d.model, d.box, d.iterations, d.camera) == (3, 15, 20, 2)
    assert list(d.psf) == pytest.approx([1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50.0, 100.0])
    assert d.lower[2] == -600 and d.upper[2] == 600 and d.max_step[2] == 60
    with pytest.raises(ValueError):
        make_desc(G.GaussianXYNB(1.3), 11, 20, simulate.ASTIG_WIDE, 0)


def test_abi_structs_have_the_header_layout(tmp_path):
    """ctypes mirrors and the C header agree on sizes and offsets (gcc-compiled probe)."""
    import subprocess
    from pathlib import Path
    inc = Path(__file__).resolve().parent.parent / "include"
    src = tmp_path / "probe.c"
    src.write_text("""
#include <stdio.h>
#include <stddef.h>
#include "gaussmle_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(gmle_fit_desc), offsetof(gmle_fit_desc, max_step),
         sizeof(gmle_group), offsetof(gmle_group, n), offsetof(gmle_group, flags),
         sizeof(gmle_server_config), sizeof(gmle_server_stats),
         offsetof(gmle_server_stats, hbm_peak_bytes));
  return 0;
}""")
    exe = tmp_path / "probe"
    subprocess.run(["gcc", "-std=c11", f"-I{inc}", str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    want = [C.sizeof(_lib.FitDesc), _lib.FitDesc.max_step.offset, C.sizeof(_lib.Group),
            _lib.Group.n.offset, _lib.Group.flags.offset, C.sizeof(_lib.ServerConfig),
            C.sizeof(_lib.ServerStats), _lib.ServerStats.hbm_peak_bytes.offset]
    assert got == want


def test_scmos_camera_maps():
    cam = G.SCMOSCamera(8, 4, 0.1, readnoise=2.0, offset=100.0, gain=0.5)
    var, gain, off = cam.calibration_maps()
    assert var.shape == (4, 8) and float(var[0, 0]) == 4.0
    assert float(gain[3, 7]) == 0.5 and float(off[0, 0]) == 100.0
    with pytest.raises(ValueError):
        G.SCMOSCamera(8, 4, 0.1, readnoise=np.ones((8, 4), np.float32)).calibration_maps()


def test_simulated_rois_follow_the_kernel_layout():
    # pixel (i = row, j = col) of ROI k at data[i, j, k]; the PSF peak follows (x, y)
    psf = G.GaussianXYNB(1.3)
    truth = np.array([[3.0, 8.0, 1e6, 0.0]], np.float32)    # x = 3 (column), y = 8 (row)
    mu = simulate.expectation(psf, truth, 11)                 # (n, col, row)
    data = np.ascontiguousarray(mu, np.float32).transpose(2, 1, 0)
    i, j = np.unravel_index(np.argmax(data[:, :, 0]), (11, 11))
    assert (i + 1, j + 1) == (8, 3)
    assert data.flags["F_CONTIGUOUS"]


def test_request_stream_sizes_and_mix():
    class P:  # minimal stand-in for HostPools
        g = [{"n": 100000}, {"n": 50000}]
        p = np.array([2 / 3, 1 / 3])
    reqs = loadgen.make_stream(P, 500000, seed=1)
    sizes = np.array([r.n for r in reqs])
    assert sizes.min() >= 50 and sizes.max() <= 50000 and sizes.sum() >= 500000
    assert all(r.lo + r.n <= P.g[r.group]["n"] for r in reqs)


def test_roofline_model_counts():
    w11 = roofline.work_per_roi(0, 11, 20, 0)
    w13 = roofline.work_per_roi(1, 13, 20, 2)
    assert w11["slots"] < w13["slots"]
    # the overlapping-pipe bound: the largest of FP32, SFU and FP64 time
    assert w11["slots"] == max(w11["fp32"], 8 * w11["sfu"], 64 * w11["fp64"])
    assert w11["issue"] == w11["fp32"] + w11["sfu"] + w11["fp64"] > w11["slots"]
    assert w11["fp32_equiv_sum"] > w11["issue"]
    assert roofline.work_per_roi(0, 11, 10, 0)["fp32"] < w11["fp32"]
    assert roofline.bytes_per_roi(0, 11, 0) == 484 + 8 + 4 * 8 + 5
    assert roofline.bytes_per_roi(1, 13, 2) == 169 * 4 * 4 + 8 + 5 * 8 + 5
    # 1 ms for 10^6 ROIs: the fraction is the bound's time over the measured time
    r = roofline.roofline(0, 11, 2, 10 ** 6, 1e-3, 152, 2070.0, 6760.0)
    assert r["bound"] == "fp32"
    w = roofline.work_per_roi(0, 11, 20, 2)
    assert abs(r["frac"] - 10 ** 6 * w["fp32"] / 1e-3 / 40.27392e12) < 1e-9
    assert abs(r["issue_unpacked_frac"] - 10 ** 6 * w["issue"] / 1e-3 / 40.27392e12) < 1e-9
    assert abs(r["achieved_tinst"] / r["peak_tinst"] - r["frac"]) < 1e-12


def test_library_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(G.GaussMLEError) as ei:
        G.Context(0)
    assert ei.value.status == 8  # GMLE_NO_DEVICE


def test_tuning_cache_applies_this_gpus_entries_and_skips_malformed_ones(tmp_path, monkeypatch):
    from gaussmle_gb300 import tuning
    cache = tmp_path / "tuning.json"
    monkeypatch.setattr(tuning, "CACHE", cache)
    monkeypatch.setattr(tuning, "_gpu_name", lambda device: "GB300")

    class FakeLib:
        def __init__(self):
            self.calls = []

        def gmle_set_tuning(self, handle, m, b, cam, tpr, rpb):
            self.calls.append((m, b, cam, tpr, rpb))
            return 0 if tpr in (1, 2, 4, 8) else 1  # the library rejects a bad shape

    class FakeCtx:
        device, handle, lib = 0, None, FakeLib()

    ctx = FakeCtx()
    assert tuning.load_cache(ctx) == 0  # no cache file
    cache.write_text(json.dumps({
        "GB300": {"0/11/1": [1, 128], "3/15/0": [2, 64], "1/9/1": [3, 32],
                  "bad key": [1, 32], "2/13/1": "x", "0/7/1": [1]},
        "another GPU": {"0/11/0": [8, 16]}}))
    assert tuning.load_cache(ctx) == 2
    assert ctx.lib.calls == [(0, 11, 1, 1, 128), (3, 15, 0, 2, 64), (1, 9, 1, 3, 32)]
    cache.write_text("[1, 2]")  # not a table
    assert tuning.load_cache(ctx) == 0
    cache.write_text("{")  # not JSON
    assert tuning.load_cache(ctx) == 0
