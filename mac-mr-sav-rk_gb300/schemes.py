"""Fused GPU time schemes behind the reference's ``make_scheme`` API.

``make_scheme(name, gamma)`` (solver/schemes/registry.py:44-53) returns a
scheme whose ``step(model, state, dt) -> Trial`` runs the whole step in one
``macsav_step`` call on the device (optionally as one CUDA graph): stage
right-hand sides, the two-column Stokes solves, the SAV scalar map, the
recombination, the stage gates and the convection at the stage nodes.  The
stage scalars are read back once per step; the exceptions and messages are
the reference's.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import StageRecord
from .core import DeviceArray, Stage, Trial
from .stokes import dptr, stream_handle

ETA = 1 - 1 / np.sqrt(2.0)  # solver/schemes/sdirk2.py:14
C3 = (0.0, 1 / 4, 4 / 5, 1.0)  # solver/schemes/sdirk3.py:13 (stage nodes)


@dataclass(frozen=True)
class SchemeInfo:
    """``solver/schemes/registry.py:14-21``."""
    order: int
    n_stages: int
    n_roots: int
    estimator_order: int | None
    pressure_semantics: str = "incremental_stage_multiplier_mean_zero"
    n_corrections: int = 0


_INFO = {  # registry.py:25-32
    "sdirk2": SchemeInfo(2, 2, 3, 2),
    "sdirk2_mrsav": SchemeInfo(2, 2, 3, 2, n_corrections=1),
    "sdirk3": SchemeInfo(3, 4, 5, 3),
    "sdirk3_mrsav": SchemeInfo(3, 4, 5, 3, n_corrections=2),
    "imex_euler": SchemeInfo(1, 1, 1, None, "euler_step_multiplier_mean_zero"),
    "imex_euler_mrsav": SchemeInfo(1, 1, 1, None, "euler_step_multiplier_mean_zero", n_corrections=1),
}
SCHEMES = tuple(_INFO)
DEFAULT_SCHEMES = ("sdirk2", "sdirk2_mrsav", "sdirk3", "sdirk3_mrsav")
_IDS = {"sdirk2_mrsav": 0, "sdirk3_mrsav": 1, "imex_euler_mrsav": 2, "sdirk2": 3, "sdirk3": 4, "imex_euler": 5}
_NODES = {"sdirk2_mrsav": (0.0, ETA), "sdirk2": (0.0, ETA), "sdirk3_mrsav": C3, "sdirk3": C3,
          "imex_euler_mrsav": (0.0,), "imex_euler": (0.0,)}
_GATE_PREFIX = {"imex_euler_mrsav": "IMEX Euler SAV residuals", "imex_euler": "IMEX Euler residual"}


def scheme_info(name: str) -> SchemeInfo:
    try:
        return _INFO[name]
    except KeyError as error:
        raise ValueError(f"Unknown scheme: {name}") from error


class FusedScheme:
    """One GPU scheme; ``step`` has the reference's Scheme.step signature."""

    def __init__(self, name: str, gamma: float = 1.0) -> None:
        scheme_info(name)
        if not np.isfinite(gamma) or gamma < 0:
            raise ValueError("gamma must be finite and nonnegative")
        self.name = name
        self.gamma = float(gamma)
        self.info = _INFO[name]
        self._id = _IDS[name]
        self.sav = name.endswith("_mrsav")
        self.last_records: list = []

    def _raise(self, code: int, rec: StageRecord, plan) -> None:
        st = rec.status
        if st == 1:
            raise ValueError("Invalid Stokes RHS")
        if st == 2:
            raise RuntimeError(f"Pressure Schur CG failed with info={rec.cg_info}")
        if st == 3:
            raise RuntimeError(f"Stokes residual={rec.stokes_residual:.3e}, divergence={rec.stokes_divergence:.3e}")
        if st == 4:
            raise RuntimeError("Negative Stokes response energy")
        if st == 5:
            raise ValueError("Invalid frozen SAV scalar inputs")
        if st == 6:
            raise RuntimeError("Invalid frozen SAV scalar denominator")
        if st == 7:
            raise RuntimeError("Nonfinite frozen SAV correction")
        if st == 8:
            prefix = _GATE_PREFIX.get(self.name, "SAV stage residuals")
            if self.name == "imex_euler":
                raise RuntimeError(f"{prefix} {rec.residual}, divergence {rec.continuity_residual}")
            raise RuntimeError(f"{prefix} {rec.residual}, {rec.scalar_residual}, divergence "
                               f"{rec.continuity_residual}")
        _lib.check(code, plan.handle)

    def step_device(self, model, x0: torch.Tensor, t: float, r0: float, dt: float, *, x1=None, emb=None,
                    pres=None, want_embedded: bool = True, forces=None):
        """One step on device data: x0 (packed, float64 CUDA) at time t with
        scalar r0.  Returns (x1, r1, records, pres, emb).  Raises like the
        reference when a stage check fails."""
        plan = model.plan
        g = model.grid
        n = self.info.n_stages
        if forces is None and not getattr(model.force, "zero", False):
            forces = torch.stack([model._dev(model.force(t + c * dt)).reshape(-1) for c in _NODES[self.name]])
            forces = forces.contiguous()
        if x1 is None:
            x1 = torch.empty(g.size, dtype=torch.float64, device=x0.device)
        if emb is None and want_embedded and n > 1:
            emb = torch.empty(g.size, dtype=torch.float64, device=x0.device)
        if pres is None:
            pres = torch.empty((n, g.np), dtype=torch.float64, device=x0.device)
        recs = (StageRecord * n)()
        r1 = C.c_double()
        lib = _lib.load()
        lib.macsav_plan_set_graph(plan.handle, 1 if getattr(model, "use_graph", False) else 0)
        code = lib.macsav_step(plan.handle, self._id, float(t), float(dt), float(model.nu), self.gamma,
                               dptr(x0), float(r0), dptr(forces) if forces is not None else None, dptr(x1),
                               dptr(emb) if emb is not None else None, dptr(pres), recs, C.byref(r1),
                               stream_handle())
        self.last_records = list(recs)
        if code != _lib.OK:
            failing = next((r for r in recs if r.status), None)
            if failing is None:
                _lib.check(code, plan.handle)
            self._raise(code, failing, plan)
        return x1, (float(r1.value) if self.sav else 0.0), recs, pres, emb

    def step(self, model, state, dt: float) -> Trial:
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError("Invalid step size")
        if self.name == "imex_euler" and not np.isfinite(state.t):
            raise ValueError("Invalid step size or state time")  # imex_euler.py:14-15
        if self.name == "imex_euler_mrsav" and not np.isfinite([state.t, state.r]).all():
            raise ValueError("Invalid step size or scalar state")  # imex_euler_mrsav.py:52-53
        g = model.grid
        x0 = model.device_vector(state).contiguous()
        x1, r1, recs, pres, emb = self.step_device(model, x0, state.t, state.r, dt)
        stages = []
        for i, rec in enumerate(recs):
            st = Stage(DeviceArray(pres[i].reshape(g.ny, g.nx)), float(rec.residual), float(rec.divergence_inf),
                       float(rec.r) if self.sav else 0.0, [], [], float(rec.scalar_residual) if self.sav else 0.0,
                       float(rec.continuity_residual), iterations=tuple(rec.iterations[:2 if self.sav else 1]))
            if self.sav:  # ScalarCorrection.record (scalar_correction.py:19-23)
                st.correction_predictor = float(rec.correction_predictor)
                st.corrections = [float(rec.corrections[k]) for k in range(rec.n_corrections)]
                st.frozen_factor = float(rec.frozen_factor)
            stages.append(st)
        new_state = model.state(state.t + dt, x1, r1)
        trial = Trial(new_state, stages, emb)
        if emb is not None:
            # <x1-emb, x1-emb>_h, <x0,x0>_h, <x1,x1>_h and emb's finiteness,
            # formed on the device inside the step (for the adaptive driver)
            norms = (C.c_double * 4)()
            _lib.check(_lib.load().macsav_step_embedded_norms(model.plan.handle, norms), model.plan.handle)
            trial.embedded_norms = tuple(float(v) for v in norms)
        return trial


def make_scheme(name: str, gamma: float = 1.0) -> FusedScheme:
    """``solver/schemes/registry.py:51-53``."""
    scheme_info(name)
    return FusedScheme(name, gamma)
