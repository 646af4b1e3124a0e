"""GaussMLEFitter / fit: the host side of the fit path, mirroring src/interface.jl.

What stays on the host is what the reference keeps around its GPU branch:
input validation (src/interface.jl:10-40), micron -> pixel conversion of the
PSF (src/psf_models.jl:311-331), the corner vectors, and after the fit the
p-values (src/interface.jl:265-275) and the camera-coordinate results
(src/roi_batch.jl:28-72).  The GPU branch itself (src/interface.jl:217-263,
:334-370, :421-457) is one call into libgaussmle_sm100a.so.  There is no CPU
device: asking for one, or running without the library or a GB300, raises.
"""
from __future__ import annotations

import ctypes as C
import weakref
from dataclasses import dataclass

import numpy as np

from . import _lib
from .camera import IdealCamera, ROIBatch, SCMOSCamera
from .constraints import ParameterConstraints, default_constraints
from .emitters import BasicSMLD, to_emitters
from .models import GaussianXYNB, PSFModel


def validate_fit_input(data: np.ndarray) -> None:
    """src/interface.jl:10-40: non-empty, square, at least 3x3, finite."""
    if data.size == 0:
        raise ValueError("Input data array is empty")
    if data.ndim != 3:
        raise ValueError(f"data must be (box, box, n), got shape {data.shape}")
    if data.shape[0] != data.shape[1]:
        raise ValueError(f"ROIs must be square, got size {data.shape[0]}x{data.shape[1]}")
    if data.shape[0] < 3:
        raise ValueError(f"ROI size must be at least 3x3, got {data.shape[0]}x{data.shape[0]}")
    if not np.all(np.isfinite(data)):
        raise ValueError("Input data contains NaN or Inf values")


def make_desc(psf_pixels: PSFModel, box: int, iterations: int,
              constraints: ParameterConstraints, camera: int,
              method: int = _lib.METHOD_NEWTON) -> _lib.FitDesc:
    """gmle_fit_desc.  method: METHOD_NEWTON (the reference's step) or
    METHOD_FISHER_LM (full-Hessian steps with Levenberg-Marquardt damping, an
    option with no reference counterpart)."""
    d = _lib.FitDesc()
    d.model = psf_pixels.model_id
    d.box = box
    d.iterations = iterations
    d.camera = camera
    d.method = method
    P = psf_pixels.nparams
    for t, v in enumerate(psf_pixels.psf_vector()):
        d.psf[t] = float(v)
    if len(constraints.lower) != P:
        raise ValueError(f"constraints have {len(constraints.lower)} entries, model needs {P}")
    for k in range(P):
        d.lower[k] = float(constraints.lower[k])
        d.upper[k] = float(constraints.upper[k])
        d.max_step[k] = float(constraints.max_step[k])
    return d


class GaussMLEFitter:
    """src/interface.jl:73-145.  `device` must be 'gpu' (or None/'auto'): this
    library is the GPU device and has no CPU fallback.  `method` is
    'newton' (the reference's per-parameter Newton step) or 'fisher_lm'
    (full-Hessian steps with Levenberg-Marquardt damping, an option with no
    reference counterpart)."""

    METHODS = {"newton": _lib.METHOD_NEWTON, "fisher_lm": _lib.METHOD_FISHER_LM}

    def __init__(self, psf_model: PSFModel = GaussianXYNB(0.13), device=None,
                 iterations: int = 20, constraints: ParameterConstraints | None = None,
                 batch_size: int = 10_000, context: _lib.Context | None = None,
                 method: str = "newton"):
        if device not in (None, "gpu", "auto", ":gpu"):
            raise ValueError(f"device {device!r}: only the GPU device is provided "
                             "(the reference's CPU path is not part of this library)")
        if method not in self.METHODS:
            raise ValueError(f"method {method!r}: one of {sorted(self.METHODS)}")
        self.method = method
        self.psf_model = psf_model
        self.iterations = int(iterations)
        # The reference builds default constraints for an 11x11 box whatever
        # the ROI size used later (src/interface.jl:140-142).
        self.constraints = constraints if constraints is not None else \
            default_constraints(psf_model, 11)
        self.batch_size = int(batch_size)
        self._ctx = context

    @property
    def context(self) -> _lib.Context:
        if self._ctx is None:
            self._ctx = _lib.default_context()
        return self._ctx


@dataclass
class LocalizationResult:
    """Fit output in ROI pixels plus camera-pixel positions (src/roi_batch.jl:9-72).

    params and uncertainties are (n, P): row r holds ROI r's parameters, the
    same memory as Julia's (P, n) column-major `results`."""
    params: np.ndarray
    uncertainties: np.ndarray
    log_likelihoods: np.ndarray
    pvalues: np.ndarray
    flags: np.ndarray
    x_camera: np.ndarray
    y_camera: np.ndarray
    frame_indices: np.ndarray
    psf_model: PSFModel
    pixel_size: float
    camera: object = None

    def __len__(self) -> int:
        return self.params.shape[0]

    def column(self, name: str) -> np.ndarray:
        return self.params[:, self.psf_model.param_names.index(name)]

    def to_emitters(self, dataset: int = 1, track_id: int = 0) -> np.ndarray:
        """Every fit as a record of the model's emitter type, in bulk
        (to_emitter, src/roi_batch.jl:125-302; gaussmle_gb300.emitters)."""
        cam = self.camera
        psx = float(cam.pixel_edges_x[1] - cam.pixel_edges_x[0]) if cam else self.pixel_size
        psy = float(cam.pixel_edges_y[1] - cam.pixel_edges_y[0]) if cam else self.pixel_size
        return to_emitters(self.psf_model.model_id, self.params, self.uncertainties,
                           self.pvalues, self.x_camera, self.y_camera, self.frame_indices,
                           psx, psy, dataset, track_id)

    def to_smld(self, dataset: int = 1) -> BasicSMLD:
        """BasicSMLD of the fits (to_smld, src/roi_batch.jl:326-353)."""
        n_frames = int(self.frame_indices.max()) if len(self.frame_indices) else 0
        meta = {"psf_model": type(self.psf_model).__name__, "n_fits": len(self)}
        return BasicSMLD(self.to_emitters(dataset), self.camera, n_frames, 1, meta)


def _pvalues(ctx: _lib.Context, llr: np.ndarray, box: int, nparams: int) -> np.ndarray:
    """1 - cdf(Chisq(box^2 - P), -2 llr) (src/interface.jl:265-275), on the GPU."""
    llr = np.ascontiguousarray(llr, dtype=np.float32)
    pv = np.empty_like(llr)
    ctx.check(ctx.lib.gmle_pvalues(ctx.handle, llr.ctypes.data_as(C.c_void_p), llr.size,
                                   box * box - nparams, pv.ctypes.data_as(C.c_void_p)))
    return pv


def _run(fitter: GaussMLEFitter, data_f: np.ndarray, psf_pixels: PSFModel, camera: int,
         xc: np.ndarray | None, yc: np.ndarray | None):
    ctx = fitter.context
    box, n = data_f.shape[0], data_f.shape[2]
    P = psf_pixels.nparams
    desc = make_desc(psf_pixels, box, fitter.iterations, fitter.constraints, camera,
                     GaussMLEFitter.METHODS[fitter.method])
    params = np.empty((n, P), np.float32)
    crlb = np.empty((n, P), np.float32)
    llr = np.empty(n, np.float32)
    flags = np.empty(n, np.uint8)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p) if a is not None else None
    st = ctx.lib.gmle_fit(ctx.handle, C.byref(desc), ptr(data_f), ptr(xc), ptr(yc), n,
                          ptr(params), ptr(crlb), ptr(llr), ptr(flags))
    ctx.check(st)
    return params, crlb, llr, flags


def fit(fitter: GaussMLEFitter, data, variance_map: np.ndarray | None = None):
    """fit(fitter, data (box, box, n) [row, col, roi]) / fit(fitter, ROIBatch).

    Mirrors src/interface.jl:177-291 (Array), :304-386 (ROIBatch{IdealCamera})
    and :389-473 (ROIBatch{SCMOSCamera}); returns a LocalizationResult."""
    if isinstance(data, ROIBatch):
        return _fit_batch(fitter, data)
    data = np.asarray(data)
    if data.ndim == 2:  # single ROI, src/interface.jl:294-301
        data = data[:, :, None]
    validate_fit_input(data)
    box, n = data.shape[0], data.shape[2]
    data_f = np.asfortranarray(data, dtype=np.float32)
    pixel_size = 0.1  # src/interface.jl:191
    psf_pixels = fitter.psf_model.to_pixel_units(pixel_size)
    xc = (1 + np.arange(n, dtype=np.int32) * box).astype(np.int32)
    yc = np.ones(n, np.int32)
    camera = _lib.CAMERA_POISSON
    if variance_map is not None:
        vm = np.asfortranarray(variance_map, dtype=np.float32)
        ctx = fitter.context
        ctx.check(ctx.lib.gmle_set_calibration(ctx.handle, vm.ctypes.data_as(C.c_void_p),
                                               None, None, vm.shape[0], vm.shape[1]))
        camera = _lib.CAMERA_SCMOS
    params, crlb, llr, flags = _run(fitter, data_f, psf_pixels, camera, xc, yc)
    pv = _pvalues(fitter.context, llr, box, psf_pixels.nparams)
    # the reference's Array path fits on a synthetic camera of ROIs side by
    # side, 0.1 micron pixels (src/interface.jl:191-215)
    cam = IdealCamera(box * n, box, pixel_size)
    return LocalizationResult(params, crlb, llr, pv, flags,
                              (xc + params[:, 0] - 1).astype(np.float32),
                              (yc + params[:, 1] - 1).astype(np.float32),
                              np.ones(n, np.int32), fitter.psf_model, pixel_size, cam)


_calibrated: dict = {}


def ensure_calibration(ctx: _lib.Context, cam: SCMOSCamera) -> bool:
    """Make the camera's maps the context's resident calibration; returns
    whether they were uploaded.  The resident maps are reused while their
    contents are unchanged: they are compared with the copy taken at upload,
    so an in-place edit of a camera's arrays, or another camera, uploads
    again (the reference uploads the maps with every batch,
    src/interface.jl:431-432)."""
    maps = [np.asfortranarray(m, np.float32) for m in cam.calibration_maps()]
    known = _calibrated.get(id(ctx))
    if known is not None and known[0]() is ctx and all(
            a.shape == b.shape and np.array_equal(a, b) for a, b in zip(known[1], maps)):
        return False
    var, gain, off = maps
    ctx.check(ctx.lib.gmle_set_calibration(
        ctx.handle, var.ctypes.data_as(C.c_void_p), gain.ctypes.data_as(C.c_void_p),
        off.ctypes.data_as(C.c_void_p), cam.ny, cam.nx))
    _calibrated[id(ctx)] = (weakref.ref(ctx), [m.copy() for m in maps])
    return True


def _fit_batch(fitter: GaussMLEFitter, batch: ROIBatch):
    data = np.asarray(batch.data)
    if data.ndim != 3 or data.shape[0] != data.shape[1] or data.size == 0:
        raise ValueError("ROIBatch data must be a non-empty (box, box, n) array")
    box, n = data.shape[0], data.shape[2]
    cam = batch.camera
    pixel_size = float(cam.pixel_edges_x[1] - cam.pixel_edges_x[0])
    psf_pixels = fitter.psf_model.to_pixel_units(pixel_size)
    data_f = np.asfortranarray(data, dtype=np.float32)
    ctx = fitter.context
    if isinstance(cam, SCMOSCamera):
        # Maps are uploaded once per (context, camera) and stay resident; the
        # ADU -> e- conversion (src/camera_models.jl:110-113) runs on the device.
        ensure_calibration(ctx, cam)
        camera = _lib.CAMERA_SCMOS_ADU
    elif isinstance(cam, IdealCamera):
        camera = _lib.CAMERA_POISSON
    else:
        raise TypeError(f"unsupported camera {type(cam).__name__}")
    params, crlb, llr, flags = _run(fitter, data_f, psf_pixels, camera,
                                    batch.x_corners, batch.y_corners)
    pv = _pvalues(fitter.context, llr, box, psf_pixels.nparams)
    return LocalizationResult(params, crlb, llr, pv, flags,
                              (batch.x_corners + params[:, 0] - 1).astype(np.float32),
                              (batch.y_corners + params[:, 1] - 1).astype(np.float32),
                              batch.frame_indices, fitter.psf_model, pixel_size, cam)
