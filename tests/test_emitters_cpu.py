"""Bulk emitter assembly and the calibration cache (host logic, no GPU).

to_emitters builds every emitter of a result at once; here it is checked
against a per-ROI restatement of the reference's to_emitter
(src/roi_batch.jl:125-302) and against the emitter types' field lists
(src/emitters.jl:45-237).
"""
import numpy as np
import pytest

from gaussmle_gb300 import emitters, fitter
from gaussmle_gb300.camera import IdealCamera, SCMOSCamera

JULIA_FIELDS = {  # src/emitters.jl, in declaration order
    0: "x y photons bg σ_x σ_y σ_photons σ_bg pvalue frame dataset track_id id",
    1: "x y photons bg σ σ_x σ_y σ_photons σ_bg σ_σ pvalue frame dataset track_id id",
    2: "x y photons bg σx σy σ_x σ_y σ_photons σ_bg σ_σx σ_σy pvalue frame dataset track_id id",
    3: "x y z photons bg σ_x σ_y σ_z σ_photons σ_bg pvalue frame dataset track_id id",
}


def one_emitter(model, p, u, pv, xcam, ycam, frame, px, py, idx):
    """to_emitter for one ROI, as src/roi_batch.jl:125-302 writes it (Float32)."""
    f = np.float32
    px, py = f(px), f(py)
    e = {"x": (f(xcam) - f(1)) * px, "y": (f(ycam) - f(1)) * py, "σ_x": f(u[0]) * px,
         "σ_y": f(u[1]) * py, "pvalue": f(pv), "frame": int(frame), "dataset": 1,
         "track_id": 0, "id": idx}
    if model == 3:
        e.update(z=f(p[2]), photons=f(p[3]), bg=f(p[4]), σ_z=f(u[2]), σ_photons=f(u[3]),
                 σ_bg=f(u[4]))
    else:
        e.update(photons=f(p[2]), bg=f(p[3]), σ_photons=f(u[2]), σ_bg=f(u[3]))
        if model == 1:
            e.update(σ=f(p[4]) * px, σ_σ=f(u[4]) * px)
        if model == 2:
            e.update(σx=f(p[4]) * px, σy=f(p[5]) * py, σ_σx=f(u[4]) * px, σ_σy=f(u[5]) * py)
    return e


@pytest.mark.parametrize("model", [0, 1, 2, 3])
def test_bulk_emitters_match_the_per_roi_construction(model):
    rng = np.random.default_rng(model)
    n, P = 300, {0: 4, 1: 5, 2: 6, 3: 5}[model]
    p = rng.uniform(0.5, 20, (n, P)).astype(np.float32)
    u = rng.uniform(0.01, 2, (n, P)).astype(np.float32)
    pv = rng.uniform(0, 1, n).astype(np.float32)
    xcam = rng.uniform(1, 2048, n).astype(np.float32)
    ycam = rng.uniform(1, 2048, n).astype(np.float32)
    frames = rng.integers(1, 500, n).astype(np.int32)
    out = emitters.to_emitters(model, p, u, pv, xcam, ycam, frames, 0.108, 0.108)
    assert list(out.dtype.names) == JULIA_FIELDS[model].split()
    for k in range(0, n, 37):
        ref = one_emitter(model, p[k], u[k], pv[k], xcam[k], ycam[k], frames[k], 0.108, 0.108,
                          k + 1)
        for name, v in ref.items():
            assert out[name][k] == v, (model, k, name)


def test_smld_of_a_result():
    n = 50
    res = fitter.LocalizationResult(
        np.ones((n, 4), np.float32), np.full((n, 4), 0.1, np.float32), np.zeros(n, np.float32),
        np.full(n, 0.5, np.float32), np.ones(n, np.uint8), np.full(n, 3.0, np.float32),
        np.full(n, 4.0, np.float32), np.arange(1, n + 1, dtype=np.int32),
        fitter.GaussianXYNB(0.13), 0.1, IdealCamera(64, 64, 0.1))
    smld = res.to_smld()
    assert smld.emitter_type == "Emitter2DFitGaussMLE"
    assert smld.n_frames == n and smld.n_datasets == 1
    assert smld.metadata == {"psf_model": "GaussianXYNB", "n_fits": n}
    np.testing.assert_array_equal(smld.emitters["x"], np.float32(2.0) * np.float32(0.1))
    np.testing.assert_array_equal(smld.emitters["id"], np.arange(1, n + 1))


class FakeLib:
    def __init__(self):
        self.uploads = 0

    def gmle_set_calibration(self, *args):
        self.uploads += 1
        return 0


class FakeCtx:
    def __init__(self):
        self.lib = FakeLib()
        self.handle = None

    def check(self, st):
        assert st == 0


def test_calibration_is_uploaded_again_when_a_map_changes_in_place():
    ctx = FakeCtx()
    rn = np.full((32, 48), 1.5, np.float32)
    cam = SCMOSCamera(48, 32, 0.1, rn, 100.0, 0.5)
    assert fitter.ensure_calibration(ctx, cam)        # first use: upload
    assert not fitter.ensure_calibration(ctx, cam)    # unchanged: resident maps reused
    rn[3, 7] = 2.0                                    # in-place edit of the camera's array
    assert fitter.ensure_calibration(ctx, cam)
    assert not fitter.ensure_calibration(ctx, cam)
    other = SCMOSCamera(48, 32, 0.1, rn.copy(), 100.0, 0.5)
    assert not fitter.ensure_calibration(ctx, other)  # another camera, same contents
    other.gain = 0.6
    assert fitter.ensure_calibration(ctx, other)
    assert ctx.lib.uploads == 3
