"""Parameter constraints, mirroring src/constraints.jl."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .models import (MODEL_ASTIG, MODEL_XYNB, MODEL_XYNBS, MODEL_XYNBSXSY, PSFModel)

INF = np.float32(np.inf)


@dataclass
class ParameterConstraints:
    """lower, upper and max_step per parameter (src/constraints.jl:5-9)."""
    lower: np.ndarray
    upper: np.ndarray
    max_step: np.ndarray

    def __post_init__(self):
        self.lower = np.asarray(self.lower, np.float32)
        self.upper = np.asarray(self.upper, np.float32)
        self.max_step = np.asarray(self.max_step, np.float32)
        if not (self.lower.shape == self.upper.shape == self.max_step.shape):
            raise ValueError("lower, upper and max_step must have one entry per parameter")


def default_constraints(psf_model: PSFModel, box_size: int) -> ParameterConstraints:
    """Per-model defaults, src/constraints.jl:16-47 (x, y upper bound box_size + 2)."""
    b = np.float32(box_size + 2)
    m = psf_model.model_id
    if m == MODEL_XYNB:
        return ParameterConstraints([-2, -2, 1, 0.01], [b, b, INF, INF], [1, 1, 100, 2])
    if m == MODEL_XYNBS:
        return ParameterConstraints([-2, -2, 1, 0.01, 0.3], [b, b, INF, INF, 5],
                                    [1, 1, 100, 2, 0.5])
    if m == MODEL_XYNBSXSY:
        return ParameterConstraints([-2, -2, 1, 0.01, 0.3, 0.3], [b, b, INF, INF, 5, 5],
                                    [1, 1, 100, 2, 0.5, 0.5])
    if m == MODEL_ASTIG:
        return ParameterConstraints([-2, -2, -1, 1, 0.01], [b, b, 1, INF, INF],
                                    [1, 1, 0.1, 100, 2])
    raise ValueError(f"unknown model {psf_model!r}")
