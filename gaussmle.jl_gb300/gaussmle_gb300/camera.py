"""Minimal mirrors of the SMLMData types the fit API takes.

GaussMLE.jl gets IdealCamera, SCMOSCamera and ROIBatch from SMLMData.jl (not
vendored in the reference); only the fields the fit path reads are mirrored:
pixel edges (-> pixel size), readnoise / gain / offset / qe, and the ROIBatch
arrays (data, 1-based corners, frame indices, camera).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class IdealCamera:
    """Poisson-only camera with square pixels of `pixel_size` microns."""
    nx: int
    ny: int
    pixel_size: float = 0.1

    @property
    def pixel_edges_x(self) -> np.ndarray:
        return np.arange(self.nx + 1, dtype=np.float32) * np.float32(self.pixel_size)

    @property
    def pixel_edges_y(self) -> np.ndarray:
        return np.arange(self.ny + 1, dtype=np.float32) * np.float32(self.pixel_size)


@dataclass(eq=False)
class SCMOSCamera:
    """sCMOS camera: per-pixel (or scalar) readnoise [e- rms], gain [e-/ADU],
    offset [ADU] and quantum efficiency; maps are (ny, nx), indexed [row = y, col = x]."""
    nx: int
    ny: int
    pixel_size: float
    readnoise: np.ndarray | float
    offset: np.ndarray | float = 0.0
    gain: np.ndarray | float = 1.0
    qe: np.ndarray | float = 1.0

    @property
    def pixel_edges_x(self) -> np.ndarray:
        return np.arange(self.nx + 1, dtype=np.float32) * np.float32(self.pixel_size)

    @property
    def pixel_edges_y(self) -> np.ndarray:
        return np.arange(self.ny + 1, dtype=np.float32) * np.float32(self.pixel_size)

    def _full(self, v) -> np.ndarray:
        a = np.asarray(v, np.float32)
        if a.ndim == 0:
            return np.full((self.ny, self.nx), a, np.float32)
        if a.shape != (self.ny, self.nx):
            raise ValueError(f"camera map has shape {a.shape}, expected {(self.ny, self.nx)}")
        return a

    def calibration_maps(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """(variance = readnoise^2, gain, offset) as full-sensor Float32 maps
        (extract_variance_map, src/interface.jl:43-55), from the camera's
        current arrays."""
        rn = self._full(self.readnoise)
        return (rn * rn, self._full(self.gain), self._full(self.offset))


@dataclass
class ROIBatch:
    """ROIs cut from camera frames: data (box, box, n) [row, col, roi],
    1-based corners of each ROI's first pixel on the camera, frame indices."""
    data: np.ndarray
    x_corners: np.ndarray
    y_corners: np.ndarray
    frame_indices: np.ndarray
    camera: IdealCamera | SCMOSCamera

    def __post_init__(self):
        self.x_corners = np.ascontiguousarray(self.x_corners, np.int32)
        self.y_corners = np.ascontiguousarray(self.y_corners, np.int32)
        self.frame_indices = np.ascontiguousarray(self.frame_indices, np.int32)

    def __len__(self) -> int:
        return self.data.shape[2]
