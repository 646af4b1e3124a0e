"""Emitter records and BasicSMLD assembly, in bulk.

The reference turns each fit into a mutable emitter struct, one ROI at a time
(to_emitter, src/roi_batch.jl:125-302), and collects them into
SMLMData.BasicSMLD (to_smld, src/roi_batch.jl:326-353).  Here every emitter of
a result is built at once, as one numpy structured array whose fields are the
emitter type's fields, in its field order, with its types (Float32 values,
Int64 metadata): src/emitters.jl:45 (Emitter2DFitGaussMLE), :97
(Emitter2DFitSigma), :153 (Emitter2DFitSigmaXY), :212 (Emitter3DFitGaussMLE).
The values are computed as the reference computes them, in Float32:
  x, y      (camera position - 1) * pixel size   [microns]
  sigmas    fitted width * pixel size            [microns]
  z         as fitted (the units of gamma and d)
  sigma_*   CRLB, spatial ones * pixel size
  pvalue    the goodness-of-fit p-value
  frame     the ROI's frame index; dataset, track_id, id as given (id = 1..n).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .models import MODEL_ASTIG, MODEL_XYNB, MODEL_XYNBS, MODEL_XYNBSXSY

_META = [("frame", "<i8"), ("dataset", "<i8"), ("track_id", "<i8"), ("id", "<i8")]

# (emitter type name, fields): value fields are Float32 (Julia's T)
EMITTER_TYPES = {
    MODEL_XYNB: ("Emitter2DFitGaussMLE",
                 ["x", "y", "photons", "bg", "σ_x", "σ_y", "σ_photons", "σ_bg", "pvalue"]),
    MODEL_XYNBS: ("Emitter2DFitSigma",
                  ["x", "y", "photons", "bg", "σ", "σ_x", "σ_y", "σ_photons", "σ_bg", "σ_σ",
                   "pvalue"]),
    MODEL_XYNBSXSY: ("Emitter2DFitSigmaXY",
                     ["x", "y", "photons", "bg", "σx", "σy", "σ_x", "σ_y", "σ_photons", "σ_bg",
                      "σ_σx", "σ_σy", "pvalue"]),
    MODEL_ASTIG: ("Emitter3DFitGaussMLE",
                  ["x", "y", "z", "photons", "bg", "σ_x", "σ_y", "σ_z", "σ_photons", "σ_bg",
                   "pvalue"]),
}


def emitter_dtype(model: int) -> np.dtype:
    """The structured dtype of the emitter type of a PSF model."""
    _, names = EMITTER_TYPES[model]
    return np.dtype([(nm, "<f4") for nm in names] + _META)


def to_emitters(model: int, params: np.ndarray, uncertainties: np.ndarray,
                pvalues: np.ndarray, x_camera: np.ndarray, y_camera: np.ndarray,
                frame_indices: np.ndarray, pixel_size_x: float, pixel_size_y: float,
                dataset: int = 1, track_id: int = 0) -> np.ndarray:
    """Every fit as an emitter record of the model's emitter type (to_emitter,
    src/roi_batch.jl:125-302, for all ROIs at once).  params and
    uncertainties are (n, P) in the model's parameter order; positions and
    sizes in ROI / camera pixels."""
    f4 = np.float32
    px, py = f4(pixel_size_x), f4(pixel_size_y)
    p = np.asarray(params, f4)
    u = np.asarray(uncertainties, f4)
    n = p.shape[0]
    out = np.empty(n, emitter_dtype(model))
    out["x"] = (np.asarray(x_camera, f4) - f4(1)) * px
    out["y"] = (np.asarray(y_camera, f4) - f4(1)) * py
    out["σ_x"] = u[:, 0] * px
    out["σ_y"] = u[:, 1] * py
    if model == MODEL_ASTIG:
        # [x, y, z, photons, bg]; z stays in the units of gamma and d
        out["z"] = p[:, 2]
        out["photons"], out["bg"] = p[:, 3], p[:, 4]
        out["σ_z"] = u[:, 2]
        out["σ_photons"], out["σ_bg"] = u[:, 3], u[:, 4]
    else:
        # [x, y, photons, bg, (σ | σx, σy)]
        out["photons"], out["bg"] = p[:, 2], p[:, 3]
        out["σ_photons"], out["σ_bg"] = u[:, 2], u[:, 3]
        if model == MODEL_XYNBS:
            out["σ"] = p[:, 4] * px
            out["σ_σ"] = u[:, 4] * px
        elif model == MODEL_XYNBSXSY:
            out["σx"], out["σy"] = p[:, 4] * px, p[:, 5] * py
            out["σ_σx"], out["σ_σy"] = u[:, 4] * px, u[:, 5] * py
    out["pvalue"] = np.asarray(pvalues, f4)
    out["frame"] = np.asarray(frame_indices, np.int64)
    out["dataset"] = dataset
    out["track_id"] = track_id
    out["id"] = np.arange(1, n + 1, dtype=np.int64)
    return out


@dataclass
class BasicSMLD:
    """SMLMData.BasicSMLD as to_smld builds it (src/roi_batch.jl:326-353):
    the emitters, the camera, the number of frames (the largest frame index),
    one dataset, and metadata with the PSF model and the number of fits."""
    emitters: np.ndarray
    camera: object
    n_frames: int
    n_datasets: int = 1
    metadata: dict = field(default_factory=dict)

    @property
    def emitter_type(self) -> str:
        for name, names in EMITTER_TYPES.values():
            if list(self.emitters.dtype.names[: len(names)]) == names:
                return name
        return "unknown"

    def __len__(self) -> int:
        return len(self.emitters)
