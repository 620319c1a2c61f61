"""Seam record types (the reference's solver/core.py:8-47) for the GPU model.

``State`` keeps the reference's fields (t, u, v, r) as host arrays, so the
drivers' ``np.isfinite(model.vector(state))`` checks work unchanged.  A state
produced on the GPU also carries its packed device vector; its host arrays are
made read-only so that cached copy cannot go stale.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

import numpy as np


@dataclass(frozen=True)
class State:
    t: float
    u: np.ndarray
    v: np.ndarray
    r: float = 0.0
    device: Any = field(default=None, compare=False, repr=False)


@dataclass
class Stage:
    """``solver/core.py:15-26``; ``pressure`` may be a ``DeviceArray``."""
    pressure: Any
    residual: float
    divergence_inf: float
    r: float = 0.0
    candidates: list = field(default_factory=list)
    root_residuals: list = field(default_factory=list)
    scalar_residual: float = 0.0
    continuity_residual: float = float("nan")
    correction_predictor: float = float("nan")
    corrections: list = field(default_factory=list)
    frozen_factor: float = float("nan")
    iterations: tuple = ()


def stage_diagnostics(stage: Stage) -> dict[str, Any]:
    """``solver/core.py:29-36``."""
    return {"r": stage.r, "candidates": stage.candidates, "root_residuals": stage.root_residuals,
            "root_count": len(stage.candidates), "residual": stage.residual,
            "scalar_residual": stage.scalar_residual, "divergence_inf": stage.divergence_inf,
            "continuity_residual": stage.continuity_residual,
            "correction_predictor": stage.correction_predictor, "corrections": stage.corrections,
            "correction_count": len(stage.corrections), "frozen_factor": stage.frozen_factor}


@dataclass
class Trial:
    """``solver/core.py:39-42``."""
    state: State
    stages: list
    embedded_velocity: Any | None = None


class DeviceArray:
    """A device-resident field that turns into a NumPy array on demand
    (``np.asarray(x)``); ``.tensor`` is the CUDA tensor itself."""

    __slots__ = ("tensor",)

    def __init__(self, tensor) -> None:
        self.tensor = tensor

    def __array__(self, dtype=None, copy=None):
        a = self.tensor.detach().cpu().numpy()
        return a.astype(dtype) if dtype is not None else a

    def numpy(self) -> np.ndarray:
        return self.__array__()

    @property
    def shape(self) -> tuple:
        return tuple(self.tensor.shape)

    @property
    def dtype(self):
        return np.float64

    def __repr__(self) -> str:
        return f"DeviceArray(shape={self.shape}, device={self.tensor.device})"
