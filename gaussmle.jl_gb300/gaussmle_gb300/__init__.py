"""gaussmle_gb300: GaussMLE.jl's batched per-ROI Gaussian MLE fit on GB300.

The hot path is libgaussmle_sm100a.so (hand-written CUDA for sm_103a behind
the C ABI in include/gaussmle_gb300.h); this package is the host-side mirror
of the reference's GaussMLEFitter / fit API (src/interface.jl) over ctypes.
"""
from .models import (GaussianXYNB, GaussianXYNBS, GaussianXYNBSXSY, AstigmaticXYZNB,
                     PSFModel, model_from_id)
from .constraints import ParameterConstraints, default_constraints
from .camera import IdealCamera, SCMOSCamera, ROIBatch
from .fitter import GaussMLEFitter, LocalizationResult, fit, make_desc
from ._lib import Context, GaussMLEError, FitDesc, load, library_path
from .device import cut_rois, fit_device, simulate_rois

__all__ = [
    "GaussianXYNB", "GaussianXYNBS", "GaussianXYNBSXSY", "AstigmaticXYZNB", "PSFModel",
    "model_from_id", "ParameterConstraints", "default_constraints", "IdealCamera",
    "SCMOSCamera", "ROIBatch", "GaussMLEFitter", "LocalizationResult", "fit", "make_desc",
    "Context", "GaussMLEError", "FitDesc", "load", "library_path", "fit_device", "cut_rois", "simulate_rois",
]
