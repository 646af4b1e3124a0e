"""Seeded synthetic ROI batches (no public dataset is involved in this path).

Noise models follow the reference simulator (src/simulator.jl:259-307):
Ideal camera: Poisson(mu).  sCMOS: Poisson(mu * qe) + Normal(0, readnoise)
in e-, then ADU = e- / gain + offset.  Camera maps are indexed like the fit
kernel, map[row = y_corner + i - 1, col = x_corner + j - 1] (the reference's
simulator uses the transposed indexing, src/simulator.jl:292-304).
The pixel expectation mu = bg + N * psf_x * psf_y uses the erf-integrated
Gaussian with pixel centres at 1..box, evaluated in float64.

Workload definitions (seed = 1000 + index):
  0  GaussianXYNB sigma 1.3 px, 11x11, 10 000 ROIs, Poisson
  1  GaussianXYNBS true sigma U(1.0, 1.8), 13x13, 1 000 000 ROIs, sCMOS 2048x2048
  2  AstigmaticXYZNB (1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50, 100), 15x15, 1 000 000, Poisson
  3  mixed batch of 2 000 000 ROIs over five (model, box) groups, sCMOS
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
from scipy.special import erf

from .camera import SCMOSCamera
from .constraints import ParameterConstraints, default_constraints
from .models import (AstigmaticXYZNB, GaussianXYNB, GaussianXYNBS, GaussianXYNBSXSY,
                     PSFModel, MODEL_ASTIG, MODEL_XYNB, MODEL_XYNBS, MODEL_XYNBSXSY)

CAMERA_POISSON, CAMERA_SCMOS, CAMERA_SCMOS_ADU = 0, 1, 2

# Astigmatic constraints for z in +-400 (src/constraints.jl:40-47 clamps z to +-1):
# +-600 as the initialisation clamp (src/unified_kernel.jl:249), step 1/10 of the range.
ASTIG_WIDE = ParameterConstraints([-2, -2, -600, 1, 0.01], [13, 13, 600, np.inf, np.inf],
                                  [1, 1, 60, 100, 2])


@dataclass
class Workload:
    """One homogeneous group: a single (model, box, camera) and its ROIs."""
    name: str
    psf: PSFModel                 # pixel units
    box: int
    camera: int
    constraints: ParameterConstraints
    data: np.ndarray              # (box, box, n) Fortran order, float32
    x_corners: np.ndarray         # int32, 1-based
    y_corners: np.ndarray
    truth: np.ndarray             # (n, P) float32, kernel parameter order
    iterations: int = 20
    maps: tuple | None = None     # (variance, gain, offset) (ny, nx) float32

    @property
    def n(self) -> int:
        return self.data.shape[2]


def _psf_1d(centre: np.ndarray, sigma: np.ndarray, box: int) -> np.ndarray:
    """(n, box) erf-integrated 1-D Gaussian at pixel indices 1..box."""
    t = np.arange(1, box + 1, dtype=np.float64)[None, :]
    c = centre.astype(np.float64)[:, None]
    s = np.sqrt(2.0) * sigma.astype(np.float64)[:, None]
    return 0.5 * (erf((t - c + 0.5) / s) - erf((t - c - 0.5) / s))


def astig_sigmas(z: np.ndarray, psf: AstigmaticXYZNB) -> tuple[np.ndarray, np.ndarray]:
    z = z.astype(np.float64)
    ux = (z - psf.gamma) / psf.d
    uy = (z + psf.gamma) / psf.d
    ax = 1 + ux ** 2 + psf.Ax * ux ** 3 + psf.Bx * ux ** 4
    ay = 1 + uy ** 2 + psf.Ay * uy ** 3 + psf.By * uy ** 4
    return psf.sx0 * np.sqrt(ax), psf.sy0 * np.sqrt(ay)


def expectation(psf: PSFModel, theta: np.ndarray, box: int) -> np.ndarray:
    """Pixel expectations as a C-order (n, box_col, box_row) float64 array, i.e.
    the memory of a Fortran (box_row, box_col, n) array."""
    th = theta.astype(np.float64)
    m = psf.model_id
    if m == MODEL_XYNB:
        sx = sy = np.full(len(th), psf.sigma)
        N, bg = th[:, 2], th[:, 3]
    elif m == MODEL_XYNBS:
        sx = sy = th[:, 4]
        N, bg = th[:, 2], th[:, 3]
    elif m == MODEL_XYNBSXSY:
        sx, sy = th[:, 4], th[:, 5]
        N, bg = th[:, 2], th[:, 3]
    else:
        sx, sy = astig_sigmas(th[:, 2], psf)
        N, bg = th[:, 3], th[:, 4]
    px = _psf_1d(th[:, 0], sx, box)   # (n, box) along columns j
    py = _psf_1d(th[:, 1], sy, box)   # (n, box) along rows i
    return bg[:, None, None] + N[:, None, None] * px[:, :, None] * py[:, None, :]


def _to_fortran(mu_c: np.ndarray) -> np.ndarray:
    """(n, box_col, box_row) C-order -> (box_row, box_col, n) Fortran view."""
    return np.ascontiguousarray(mu_c, np.float32).transpose(2, 1, 0)


def scmos_maps(rng: np.random.Generator, ny: int = 2048, nx: int = 2048):
    """Lognormal read-noise variance (median 2 e-^2, sigma_log 0.5), gain
    U(0.4, 0.6) e-/ADU, offset 100 ADU; (ny, nx) Fortran float32."""
    var = np.exp(np.log(2.0) + 0.5 * rng.standard_normal((ny, nx))).astype(np.float32)
    gain = rng.uniform(0.4, 0.6, (ny, nx)).astype(np.float32)
    off = np.full((ny, nx), 100.0, np.float32)
    return np.asfortranarray(var), np.asfortranarray(gain), np.asfortranarray(off)


def poisson_rois(rng, psf, theta, box) -> np.ndarray:
    mu = expectation(psf, theta, box)
    return _to_fortran(rng.poisson(mu).astype(np.float32))


def scmos_rois(rng, psf, theta, box, maps, xc, yc, qe: float = 1.0) -> np.ndarray:
    """ADU data of ROIs at 1-based corners (xc, yc) on the maps' sensor."""
    var, gain, off = maps
    mu = expectation(psf, theta, box) * qe
    e = rng.poisson(mu).astype(np.float64)
    j = np.arange(box)[None, :, None]
    i = np.arange(box)[None, None, :]
    rows = (yc.astype(np.int64)[:, None, None] - 1) + i
    cols = (xc.astype(np.int64)[:, None, None] - 1) + j
    v = var[rows, cols].astype(np.float64)
    g = gain[rows, cols].astype(np.float64)
    o = off[rows, cols].astype(np.float64)
    e = e + rng.standard_normal(e.shape) * np.sqrt(v)
    return _to_fortran(e / g + o)


def random_corners(rng, n, box, ny, nx):
    xc = rng.integers(1, nx - box + 2, n).astype(np.int32)
    yc = rng.integers(1, ny - box + 2, n).astype(np.int32)
    return xc, yc


def _xy_n_bg(rng, n, box, nlo=500.0, nhi=5000.0, blo=1.0, bhi=20.0, log_n=False):
    c = (box + 1) / 2.0
    x = rng.uniform(c - 1.5, c + 1.5, n)
    y = rng.uniform(c - 1.5, c + 1.5, n)
    N = np.exp(rng.uniform(np.log(nlo), np.log(nhi), n)) if log_n else rng.uniform(nlo, nhi, n)
    bg = rng.uniform(blo, bhi, n)
    return x, y, N, bg


def xynb11_poisson(n: int = 10_000, seed: int = 1000) -> Workload:
    rng = np.random.Generator(np.random.Philox(seed))
    box, psf = 11, GaussianXYNB(1.3)
    x, y, N, bg = _xy_n_bg(rng, n, box)
    truth = np.stack([x, y, N, bg], 1).astype(np.float32)
    data = poisson_rois(rng, psf, truth, box)
    ones = np.ones(n, np.int32)
    return Workload("xynb-11-poisson", psf, box, CAMERA_POISSON, default_constraints(psf, 11),
                    data, ones, ones, truth)


def xynbs13_scmos(n: int = 1_000_000, seed: int = 1001, sensor: int = 2048) -> Workload:
    rng = np.random.Generator(np.random.Philox(seed))
    box, psf = 13, GaussianXYNBS()
    maps = scmos_maps(rng, sensor, sensor)
    x, y, N, bg = _xy_n_bg(rng, n, box)
    s = rng.uniform(1.0, 1.8, n)
    truth = np.stack([x, y, N, bg, s], 1).astype(np.float32)
    xc, yc = random_corners(rng, n, box, sensor, sensor)
    data = scmos_rois(rng, psf, truth, box, maps, xc, yc)
    return Workload("xynbs-13-scmos", psf, box, CAMERA_SCMOS_ADU, default_constraints(psf, 11),
                    data, xc, yc, truth, maps=maps)


def astig15_poisson(n: int = 1_000_000, seed: int = 1002) -> Workload:
    rng = np.random.Generator(np.random.Philox(seed))
    box = 15
    psf = AstigmaticXYZNB(1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50.0, 100.0)
    x, y, N, bg = _xy_n_bg(rng, n, box, 1000, 10000, 2, 30)
    z = rng.uniform(-400, 400, n)
    truth = np.stack([x, y, z, N, bg], 1).astype(np.float32)
    data = poisson_rois(rng, psf, truth, box)
    ones = np.ones(n, np.int32)
    return Workload("astig-15-poisson", psf, box, CAMERA_POISSON, ASTIG_WIDE, data, ones, ones,
                    truth)


# Mixed batch: (fraction, model, box).
MIX = [(0.40, MODEL_XYNB, 11), (0.25, MODEL_XYNBS, 9), (0.15, MODEL_XYNBSXSY, 13),
       (0.15, MODEL_ASTIG, 15), (0.05, MODEL_XYNB, 7)]


def mixed_group(rng, model: int, box: int, n: int, maps, sensor: int) -> Workload:
    x, y, N, bg = _xy_n_bg(rng, n, box, 100, 20000, 1, 20, log_n=True)
    if model == MODEL_XYNB:
        psf = GaussianXYNB(1.3)
        truth = np.stack([x, y, N, bg], 1)
        cons = default_constraints(psf, 11)
    elif model == MODEL_XYNBS:
        psf = GaussianXYNBS()
        truth = np.stack([x, y, N, bg, rng.uniform(1.0, 1.8, n)], 1)
        cons = default_constraints(psf, 11)
    elif model == MODEL_XYNBSXSY:
        psf = GaussianXYNBSXSY()
        truth = np.stack([x, y, N, bg, rng.uniform(1, 2, n), rng.uniform(1, 2, n)], 1)
        cons = default_constraints(psf, 11)
    else:
        psf = AstigmaticXYZNB(1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50.0, 100.0)
        truth = np.stack([x, y, rng.uniform(-400, 400, n), N, bg], 1)
        cons = ASTIG_WIDE
    truth = truth.astype(np.float32)
    xc, yc = random_corners(rng, n, box, sensor, sensor)
    data = scmos_rois(rng, psf, truth, box, maps, xc, yc)
    return Workload(f"m{model}-{box}-scmos", psf, box, CAMERA_SCMOS_ADU, cons, data, xc, yc,
                    truth, maps=maps)


def mixed_batch_scmos(n: int = 2_000_000, seed: int = 1003, sensor: int = 2048) -> list[Workload]:
    rng = np.random.Generator(np.random.Philox(seed))
    maps = scmos_maps(rng, sensor, sensor)
    counts = [int(round(f * n)) for f, _, _ in MIX]
    counts[0] += n - sum(counts)
    return [mixed_group(rng, m, b, c, maps, sensor) for (_, m, b), c in zip(MIX, counts)]


def generate_roi_batch(camera, psf_microns: PSFModel, n_rois: int, roi_size: int,
                       true_params: np.ndarray, corners: np.ndarray, seed: int = 42):
    """Mirror of generate_roi_batch (src/simulator.jl:35-108) for tests: ROIs of
    a camera at explicit 1-based corners (2, n) [x; y]; true_params (n, P) in
    ROI pixels; returns ROIBatch data in ADU for an SCMOSCamera."""
    from .camera import ROIBatch
    rng = np.random.Generator(np.random.Philox(seed))
    psf = psf_microns.to_pixel_units(camera.pixel_size)
    xc = np.asarray(corners[0], np.int32)
    yc = np.asarray(corners[1], np.int32)
    if isinstance(camera, SCMOSCamera):
        maps = camera.calibration_maps()
        qe = float(np.asarray(camera.qe).mean())
        data = scmos_rois(rng, psf, true_params, roi_size, maps, xc, yc, qe)
    else:
        data = poisson_rois(rng, psf, true_params, roi_size)
    return ROIBatch(data, xc, yc, np.ones(n_rois, np.int32), camera)


# ---- on-device generation (benchmark inputs at 10^6 ROIs) --------------------

def _poisson_t(torch, mu, g):
    """torch.poisson on the device, after a host-side check that every rate is
    finite and >= 0: torch's kernel stops the device on an invalid rate (a
    device-side assert), the check raises an exception instead."""
    bad = int((~torch.isfinite(mu) | (mu < 0)).sum().item())
    if bad:
        raise RuntimeError(f"{bad} of {mu.numel()} Poisson rates are negative or not finite")
    return torch.poisson(mu, generator=g)


def _psf_1d_t(torch, centre, sigma, box):
    t = torch.arange(1, box + 1, dtype=torch.float64, device=centre.device)[None, :]
    c = centre.double()[:, None]
    s = (2.0 ** 0.5) * sigma.double()[:, None]
    return 0.5 * (torch.special.erf((t - c + 0.5) / s) - torch.special.erf((t - c - 0.5) / s))


def xynbs13_scmos_device(n: int = 1_000_000, seed: int = 1001, sensor: int = 2048, device="cuda"):
    """XYNBS 13x13 sCMOS ADU ROIs at random corners of 2048x2048 maps,
    generated with torch on the device (the distributions of xynbs13_scmos();
    a different random stream).  Returns a dict of device tensors:
    data (n*13*13 ROI-major, Julia (box, box, n) layout), xc, yc, var, gain,
    offset ((ny, nx) column-major = tensors of shape (nx, ny)), truth (n, 5)."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    f64 = dict(dtype=torch.float64, device=device)
    box = 13
    # maps stored column-major (ny, nx): a row-major (nx, ny) tensor
    var = torch.exp(np.log(2.0) + 0.5 * torch.randn((sensor, sensor), generator=g, **f64)).float()
    gain = (0.4 + 0.2 * torch.rand((sensor, sensor), generator=g, **f64)).float()
    off = torch.full((sensor, sensor), 100.0, dtype=torch.float32, device=device)
    c = (box + 1) / 2.0
    u = lambda lo, hi: lo + (hi - lo) * torch.rand(n, generator=g, **f64)
    x, y, N, bg, s = u(c - 1.5, c + 1.5), u(c - 1.5, c + 1.5), u(500, 5000), u(1, 20), u(1.0, 1.8)
    truth = torch.stack([x, y, N, bg, s], 1).float()
    xc = torch.randint(1, sensor - box + 2, (n,), generator=g, device=device, dtype=torch.int32)
    yc = torch.randint(1, sensor - box + 2, (n,), generator=g, device=device, dtype=torch.int32)
    px = _psf_1d_t(torch, x, s, box)                      # (n, box) columns j
    py = _psf_1d_t(torch, y, s, box)                      # (n, box) rows i
    mu = bg[:, None, None] + N[:, None, None] * px[:, :, None] * py[:, None, :]  # (n, j, i)
    e = _poisson_t(torch, mu, g)
    jj = torch.arange(box, device=device)[None, :, None]
    ii = torch.arange(box, device=device)[None, None, :]
    cols = (xc.long()[:, None, None] - 1) + jj
    rows = (yc.long()[:, None, None] - 1) + ii
    v = var[cols, rows].double()      # (nx, ny) storage: [col, row]
    gg = gain[cols, rows].double()
    oo = off[cols, rows].double()
    e = e + torch.randn(e.shape, generator=g, **f64) * v.sqrt()
    data = (e / gg + oo).float().contiguous().view(-1)
    return {"data": data, "xc": xc, "yc": yc, "var": var, "gain": gain, "offset": off,
            "truth": truth, "box": box, "n": n, "ny": sensor, "nx": sensor}


def device_workload(model: int, box: int, camera: int, n: int, seed: int = 2024,
                    sensor: int = 2048, device="cuda"):
    """A homogeneous on-device batch of any (model, box, camera) with the
    distributions of the mixed workload (x, y within +-1.5 px of the centre,
    N U(500, 5000), bg U(1, 20); sigma U(1.0, 1.8); sigma_x, sigma_y U(1, 2);
    astigmatic z U(-400, 400) with the (1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50,
    100) calibration).  Same return layout as xynbs13_scmos_device()."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    f64 = dict(dtype=torch.float64, device=device)
    c = (box + 1) / 2.0
    u = lambda lo, hi: lo + (hi - lo) * torch.rand(n, generator=g, **f64)
    x, y, N, bg = u(c - 1.5, c + 1.5), u(c - 1.5, c + 1.5), u(500, 5000), u(1, 20)
    if model == MODEL_XYNB:
        psf = GaussianXYNB(1.3)
        sx = sy = torch.full((n,), 1.3, **f64)
        truth = torch.stack([x, y, N, bg], 1)
    elif model == MODEL_XYNBS:
        psf = GaussianXYNBS()
        sx = sy = u(1.0, 1.8)
        truth = torch.stack([x, y, N, bg, sx], 1)
    elif model == MODEL_XYNBSXSY:
        psf = GaussianXYNBSXSY()
        sx, sy = u(1.0, 2.0), u(1.0, 2.0)
        truth = torch.stack([x, y, N, bg, sx, sy], 1)
    else:
        psf = AstigmaticXYZNB(1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50.0, 100.0)
        z = u(-400, 400)
        zx, zy = (z - psf.gamma) / psf.d, (z + psf.gamma) / psf.d
        sx = psf.sx0 * torch.sqrt(1 + zx ** 2 + psf.Ax * zx ** 3 + psf.Bx * zx ** 4)
        sy = psf.sy0 * torch.sqrt(1 + zy ** 2 + psf.Ay * zy ** 3 + psf.By * zy ** 4)
        truth = torch.stack([x, y, z, N, bg], 1)
    px = _psf_1d_t(torch, x, sx, box)
    py = _psf_1d_t(torch, y, sy, box)
    mu = bg[:, None, None] + N[:, None, None] * px[:, :, None] * py[:, None, :]
    e = _poisson_t(torch, mu, g)
    out = {"truth": truth.float(), "box": box, "n": n, "psf": psf, "model": model,
           "camera": camera, "ny": 0, "nx": 0, "xc": None, "yc": None}
    if camera:
        var = torch.exp(np.log(2.0) + 0.5 * torch.randn((sensor, sensor), generator=g, **f64)).float()
        gain = (0.4 + 0.2 * torch.rand((sensor, sensor), generator=g, **f64)).float()
        off = torch.full((sensor, sensor), 100.0, dtype=torch.float32, device=device)
        xc = torch.randint(1, sensor - box + 2, (n,), generator=g, device=device, dtype=torch.int32)
        yc = torch.randint(1, sensor - box + 2, (n,), generator=g, device=device, dtype=torch.int32)
        jj = torch.arange(box, device=device)[None, :, None]
        ii = torch.arange(box, device=device)[None, None, :]
        cols = (xc.long()[:, None, None] - 1) + jj
        rows = (yc.long()[:, None, None] - 1) + ii
        v = var[cols, rows].double()
        e = e + torch.randn(e.shape, generator=g, **f64) * v.sqrt()
        if camera == CAMERA_SCMOS_ADU:
            e = e / gain[cols, rows].double() + off[cols, rows].double()
        out.update(var=var, gain=gain, offset=off, xc=xc, yc=yc, ny=sensor, nx=sensor)
    out["data"] = e.float().contiguous().view(-1)
    return out


def mixed_batch_scmos_device(n: int = 2_000_000, seed: int = 1003, sensor: int = 2048, device="cuda"):
    """The mixed batch on the device: n ROIs in the MIX proportions
    (40% XYNB 11x11, 25% XYNBS 9x9, 15% XYNBSXSY 13x13 with sigma_x, sigma_y
    U(1, 2), 15% astigmatic 15x15, 5% XYNB 7x7), N log-uniform 100..20000,
    bg U(1, 20), sCMOS ADU data on one shared 2048x2048 calibration map set.
    Returns (maps dict, list of group dicts like device_workload())."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    f64 = dict(dtype=torch.float64, device=device)
    var = torch.exp(np.log(2.0) + 0.5 * torch.randn((sensor, sensor), generator=g, **f64)).float()
    gain = (0.4 + 0.2 * torch.rand((sensor, sensor), generator=g, **f64)).float()
    off = torch.full((sensor, sensor), 100.0, dtype=torch.float32, device=device)
    maps = {"var": var, "gain": gain, "offset": off, "ny": sensor, "nx": sensor}
    counts = [int(round(f * n)) for f, _, _ in MIX]
    counts[0] += n - sum(counts)
    groups = []
    for (frac, model, box), cnt in zip(MIX, counts):
        c = (box + 1) / 2.0
        u = lambda lo, hi: lo + (hi - lo) * torch.rand(cnt, generator=g, **f64)
        x, y, bg = u(c - 1.5, c + 1.5), u(c - 1.5, c + 1.5), u(1, 20)
        N = torch.exp(u(np.log(100.0), np.log(20000.0)))
        if model == MODEL_XYNB:
            psf, cons = GaussianXYNB(1.3), default_constraints(GaussianXYNB(1.3), 11)
            sx = sy = torch.full((cnt,), 1.3, **f64)
            truth = torch.stack([x, y, N, bg], 1)
        elif model == MODEL_XYNBS:
            psf = GaussianXYNBS()
            cons = default_constraints(psf, 11)
            sx = sy = u(1.0, 1.8)
            truth = torch.stack([x, y, N, bg, sx], 1)
        elif model == MODEL_XYNBSXSY:
            psf = GaussianXYNBSXSY()
            cons = default_constraints(psf, 11)
            sx, sy = u(1.0, 2.0), u(1.0, 2.0)
            truth = torch.stack([x, y, N, bg, sx, sy], 1)
        else:
            psf = AstigmaticXYZNB(1.3, 1.3, 0.05, 0.05, 0.3, 0.3, 50.0, 100.0)
            cons = ASTIG_WIDE
            z = u(-400, 400)
            zx, zy = (z - psf.gamma) / psf.d, (z + psf.gamma) / psf.d
            sx = psf.sx0 * torch.sqrt(1 + zx ** 2 + psf.Ax * zx ** 3 + psf.Bx * zx ** 4)
            sy = psf.sy0 * torch.sqrt(1 + zy ** 2 + psf.Ay * zy ** 3 + psf.By * zy ** 4)
            truth = torch.stack([x, y, z, N, bg], 1)
        px = _psf_1d_t(torch, x, sx, box)
        py = _psf_1d_t(torch, y, sy, box)
        mu = bg[:, None, None] + N[:, None, None] * px[:, :, None] * py[:, None, :]
        e = _poisson_t(torch, mu, g)
        xc = torch.randint(1, sensor - box + 2, (cnt,), generator=g, device=device, dtype=torch.int32)
        yc = torch.randint(1, sensor - box + 2, (cnt,), generator=g, device=device, dtype=torch.int32)
        jj = torch.arange(box, device=device)[None, :, None]
        ii = torch.arange(box, device=device)[None, None, :]
        cols = (xc.long()[:, None, None] - 1) + jj
        rows = (yc.long()[:, None, None] - 1) + ii
        e = e + torch.randn(e.shape, generator=g, **f64) * var[cols, rows].double().sqrt()
        e = e / gain[cols, rows].double() + off[cols, rows].double()
        groups.append({"data": e.float().contiguous().view(-1), "xc": xc, "yc": yc,
                       "truth": truth.float(), "box": box, "n": cnt, "psf": psf, "model": model,
                       "camera": CAMERA_SCMOS_ADU, "constraints": cons})
    return maps, groups
