"""PSF models, mirroring src/psf_models.jl.

Widths are given in microns, as in the reference; ``to_pixel_units``
(src/psf_models.jl:311-331) converts them for the kernel.  The astigmatic
gamma and d stay in their own (physical) units: z is not converted.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

MODEL_XYNB, MODEL_XYNBS, MODEL_XYNBSXSY, MODEL_ASTIG = 0, 1, 2, 3


class PSFModel:
    model_id: int = -1
    nparams: int = 0
    param_names: tuple = ()

    def __len__(self) -> int:
        return self.nparams

    def psf_vector(self) -> np.ndarray:
        """The 8 model constants the C ABI takes (pixel units)."""
        return np.zeros(8, np.float32)


@dataclass(frozen=True)
class GaussianXYNB(PSFModel):
    """Fixed-width Gaussian, parameters [x, y, N, bg] (src/psf_models.jl:39-41)."""
    sigma: float = 0.13  # microns
    model_id = MODEL_XYNB
    nparams = 4
    param_names = ("x", "y", "photons", "bg")

    def to_pixel_units(self, pixel_size: float) -> "GaussianXYNB":
        return GaussianXYNB(float(np.float32(self.sigma) / np.float32(pixel_size)))

    def psf_vector(self) -> np.ndarray:
        v = np.zeros(8, np.float32)
        v[0] = self.sigma
        return v


@dataclass(frozen=True)
class GaussianXYNBS(PSFModel):
    """Fitted isotropic width, parameters [x, y, N, bg, sigma] (src/psf_models.jl:64)."""
    model_id = MODEL_XYNBS
    nparams = 5
    param_names = ("x", "y", "photons", "bg", "sigma")

    def to_pixel_units(self, pixel_size: float) -> "GaussianXYNBS":
        return self


@dataclass(frozen=True)
class GaussianXYNBSXSY(PSFModel):
    """Fitted sigma_x, sigma_y, parameters [x, y, N, bg, sx, sy] (src/psf_models.jl:91)."""
    model_id = MODEL_XYNBSXSY
    nparams = 6
    param_names = ("x", "y", "photons", "bg", "sigma_x", "sigma_y")

    def to_pixel_units(self, pixel_size: float) -> "GaussianXYNBSXSY":
        return self


@dataclass(frozen=True)
class AstigmaticXYZNB(PSFModel):
    """Astigmatic 3-D PSF, parameters [x, y, z, N, bg] (src/psf_models.jl:141-154).

    sigma_x(z) = sx0 * sqrt(1 + u^2 + Ax u^3 + Bx u^4), u = (z - gamma)/d;
    sigma_y(z) likewise with z + gamma.
    """
    sx0: float = 0.13
    sy0: float = 0.13
    Ax: float = 0.05
    Ay: float = 0.05
    Bx: float = 0.3
    By: float = 0.3
    gamma: float = 0.05
    d: float = 0.4
    model_id = MODEL_ASTIG
    nparams = 5
    param_names = ("x", "y", "z", "photons", "bg")

    def to_pixel_units(self, pixel_size: float) -> "AstigmaticXYZNB":
        px = np.float32(pixel_size)
        return AstigmaticXYZNB(float(np.float32(self.sx0) / px), float(np.float32(self.sy0) / px),
                               self.Ax, self.Ay, self.Bx, self.By, self.gamma, self.d)

    def psf_vector(self) -> np.ndarray:
        return np.array([self.sx0, self.sy0, self.Ax, self.Ay, self.Bx, self.By,
                         self.gamma, self.d], np.float32)


def model_from_id(model_id: int, psf: np.ndarray | None = None) -> PSFModel:
    """A pixel-unit model from the ABI's (model id, psf[8]) pair."""
    psf = np.zeros(8, np.float32) if psf is None else np.asarray(psf, np.float32)
    if model_id == MODEL_XYNB:
        return GaussianXYNB(float(psf[0]))
    if model_id == MODEL_XYNBS:
        return GaussianXYNBS()
    if model_id == MODEL_XYNBSXSY:
        return GaussianXYNBSXSY()
    if model_id == MODEL_ASTIG:
        return AstigmaticXYZNB(*[float(v) for v in psf])
    raise ValueError(f"unknown model id {model_id}")
