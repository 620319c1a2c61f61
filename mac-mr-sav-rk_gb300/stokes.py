"""GPU ``TensorStokes`` backend: the reference's StokesBackend on the CUDA library.

Drop-in for ``solver.mac.tensor_stokes.TensorStokes`` (tensor_stokes.py:118-364):
same constructor controls, ``solve(rhs, *, mass, viscosity) -> StokesResult``,
same exceptions and messages, same counters.  NumPy input gives NumPy output
(host copies inside the call); a CUDA ``torch.Tensor`` input stays on the
device.  The work runs on the current torch CUDA stream and is synchronised
before ``solve`` returns.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from time import perf_counter
from typing import Any

import numpy as np
import torch

from . import _lib
from .grid import MACGrid, grid_of

PRECISIONS = {"fp64": _lib.FP64, "fp32": _lib.FP32_MIXED, "fp32_mixed": _lib.FP32_MIXED}
# launch-shape autotuner (macsav_plan_autotune_launch_shapes): pass kinds and shapes
SHAPE_KINDS = ("velocity_rows_forward", "velocity_columns", "velocity_rows_inverse", "pressure_rows_forward",
               "pressure_columns", "pressure_rows_inverse")
SHAPE_NAMES = ("rule", "plain", "doubled", "split")


@dataclass
class StokesResult:
    """``solver/mac/stokes.py:32-37``."""
    velocity: Any
    pressure: Any
    residual: float
    divergence_inf: float


def stream_handle() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def dptr(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


class Plan:
    """Owns one ``macsav_plan`` (tables + device work buffers) for a grid."""

    def __init__(self, grid: MACGrid, precision: str = "fp64", tolerance: float = 1e-9,
                 krylov_tolerance: float = 1e-12, max_iterations: int = 100, max_columns: int = 2,
                 autotune: bool = False) -> None:
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (the GB300 library has no CPU fallback)")
        self.lib = _lib.load()
        self.grid = grid
        self.precision = precision
        handle = C.c_void_p()
        torch.cuda.init()
        code = self.lib.macsav_plan_create(C.byref(handle), grid.nx, grid.ny, float(grid.lx), float(grid.ly),
                                           PRECISIONS[precision], float(tolerance), float(krylov_tolerance),
                                           int(max_iterations), int(max_columns))
        if code != _lib.OK:
            _lib.check(code, None)
        self.handle = handle
        self.max_columns = max_columns
        # opt-in: time the transform passes' launch shapes once (tens of
        # milliseconds; the results do not change).  It times stand-alone
        # passes with plain sources and sinks; measured on GB300 at 1024^2 its
        # picks (plain forward velocity rows, doubled forward pressure rows)
        # left the step 1 % slower than the plans' rule (6.99 vs 6.92 ms), so
        # plans keep the rule unless asked.
        self.launch_shapes = self.autotune_launch_shapes() if autotune else None

    def __del__(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                torch.cuda.synchronize()
            except Exception:
                pass
            self.lib.macsav_plan_destroy(h)
            self.handle = None

    def autotune_launch_shapes(self, reps: int = 20) -> dict[str, str]:
        """Time and keep the fastest launch shape per transform pass kind
        (FP32 plans); returns the kept shape per kind."""
        chosen = (C.c_int * 6)()
        self.check(self.lib.macsav_plan_autotune_launch_shapes(self.handle, int(reps), chosen, stream_handle()))
        return {k: SHAPE_NAMES[c] for k, c in zip(SHAPE_KINDS, chosen)}

    @property
    def launches(self) -> int:
        return int(self.lib.macsav_plan_launches(self.handle))

    def check(self, code: int) -> None:
        _lib.check(code, self.handle)


def _as_device_columns(rhs, size: int) -> tuple[torch.Tensor, bool, bool]:
    """(c, size) contiguous float64 CUDA tensor, plus (was 2-D, was torch)."""
    is_torch = isinstance(rhs, torch.Tensor)
    arr = rhs if is_torch else np.asarray(rhs)
    if arr.ndim not in (1, 2) or arr.shape[0] != size:
        raise ValueError("Invalid Stokes RHS")
    two_d = arr.ndim == 2
    if is_torch:
        t = rhs.to(device="cuda", dtype=torch.float64)
    else:
        t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64)).to("cuda", non_blocking=False)
    t = (t.T if two_d else t[None, :]).contiguous()
    return t, two_d, is_torch


class TensorStokes:
    """No-slip MAC Stokes backend on one GB300 (see module docstring)."""

    def __init__(self, operators, tolerance: float = 1e-9, krylov_tolerance: float = 1e-12,
                 max_iterations: int = 100, matrix_free_operators: bool = True,
                 reuse_transform_buffers: bool = True, *, precision: str = "fp64", max_columns: int = 2,
                 corrections: int | None = None, inner_krylov_tolerance: float | None = None,
                 first_krylov_tolerance: float | None = None, autotune_launch_shapes: bool = False) -> None:
        # tensor_stokes.py:137-147
        if (tolerance <= 0 or krylov_tolerance <= 0 or not np.isfinite([tolerance, krylov_tolerance]).all()
                or max_iterations < 1):
            raise ValueError("Invalid solver controls")
        if not isinstance(matrix_free_operators, bool):
            raise ValueError("matrix_free_operators must be a bool")
        if not isinstance(reuse_transform_buffers, bool):
            raise ValueError("reuse_transform_buffers must be a bool")
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        start = perf_counter()
        self.ops = operators
        self.grid = grid_of(operators)
        self.tolerance = tolerance
        self.krylov_tolerance = krylov_tolerance
        self.max_iterations = max_iterations
        self.matrix_free_operators = matrix_free_operators
        self.reuse_transform_buffers = reuse_transform_buffers
        self.precision = precision
        self.plan = Plan(self.grid, precision, tolerance, krylov_tolerance, max_iterations,
                         max(2, min(max_columns, _lib.MAX_COLUMNS)), autotune=autotune_launch_shapes)
        if corrections is not None or inner_krylov_tolerance is not None:
            # FP32-bulk defect correction: sweeps after the first FP32 solve and
            # the inner FP32 Krylov tolerance (the FP64 closing gates stay as-is)
            self.plan.check(self.plan.lib.macsav_plan_set_refinement(
                self.plan.handle, 2 if corrections is None else int(corrections),
                1e-4 if inner_krylov_tolerance is None else float(inner_krylov_tolerance)))
        if first_krylov_tolerance is not None:
            self.plan.check(self.plan.lib.macsav_plan_set_first_solve_tolerance(self.plan.handle,
                                                                               float(first_krylov_tolerance)))
        self.setup_seconds = perf_counter() - start
        self.solve_seconds = 0.0
        self.solves = 0
        self.right_hand_sides = 0
        self.total_iterations = 0
        self.last_iterations: tuple[int, ...] = ()
        self.last_refinements = 0

    def solve_device(self, f: torch.Tensor, mass: float, viscosity: float,
                     velocity: torch.Tensor | None = None, pressure: torch.Tensor | None = None):
        """Column-blocked device solve: f is (c, size) float64 CUDA; returns
        (velocity (c, size), pressure (c, np), info).  Raises like the reference."""
        g = self.grid
        c = f.shape[0]
        if c > self.plan.max_columns:
            raise ValueError(f"at most {self.plan.max_columns} right-hand sides per solve")
        if velocity is None:
            velocity = torch.empty((c, g.size), dtype=torch.float64, device=f.device)
        if pressure is None:
            pressure = torch.empty((c, g.np), dtype=torch.float64, device=f.device)
        info = _lib.StokesInfo()
        code = self.plan.lib.macsav_stokes_solve(self.plan.handle, dptr(f), c, float(mass), float(viscosity),
                                                 dptr(velocity), dptr(pressure), C.byref(info), stream_handle())
        iters = tuple(int(info.iterations[k]) for k in range(c))
        if code == _lib.OK or code in (_lib.ERR_STOKES_GATE,):
            self.solves += 1
            self.right_hand_sides += c
            self.total_iterations += sum(iters)
            self.last_iterations = iters
            self.last_refinements = int(info.refinements)
        self.plan.check(code)
        return velocity, pressure, info

    def _spectral(self, which: int, values, size: int, mass: float, viscosity: float):
        f, two_d, is_torch = _as_device_columns(values, size)
        if f.shape[0] > self.plan.max_columns:
            raise ValueError(f"at most {self.plan.max_columns} columns per call")
        out = torch.empty_like(f)
        fn = self.plan.lib.macsav_velocity_inverse if which == 0 else self.plan.lib.macsav_schur_precondition
        self.plan.check(fn(self.plan.handle, dptr(f), dptr(out), f.shape[0], float(mass), float(viscosity),
                           stream_handle()))
        res = out.T if two_d else out[0]
        return res if is_torch else res.cpu().numpy().copy()

    def velocity_inverse(self, values, mass: float, viscosity: float):
        """(mass I + viscosity K)^{-1} of packed velocity columns in the
        solver's precision (``TensorStokes._velocity_inverse`` with the shifts
        mass + viscosity * eigenvalues, tensor_stokes.py:200-215)."""
        return self._spectral(0, values, self.grid.size, mass, viscosity)

    def precondition(self, pressure, mass: float, viscosity: float):
        """The pressure Schur CG preconditioner mass (D D^T)^+ p + viscosity p
        on the mean-zero part of cell columns, mean zero (the ``precondition``
        closure of ``TensorStokes.solve``, tensor_stokes.py:217-243,281-287)."""
        return self._spectral(1, pressure, self.grid.np, mass, viscosity)

    def solve(self, rhs, *, mass: float, viscosity: float) -> StokesResult:
        """``TensorStokes.solve`` (tensor_stokes.py:245-364)."""
        if not np.isfinite([mass, viscosity]).all() or min(mass, viscosity) < 0 or mass + viscosity <= 0:
            raise ValueError("Require mass,viscosity >= 0 and nonzero total")
        start = perf_counter()
        g = self.grid
        f, two_d, is_torch = _as_device_columns(rhs, g.size)
        try:
            vel, pres, info = self.solve_device(f, mass, viscosity)
        finally:
            self.solve_seconds += perf_counter() - start
        if is_torch:
            velocity = vel.T if two_d else vel[0]
            pressure = pres.reshape(-1, g.ny, g.nx).permute(1, 2, 0) if two_d else pres[0].reshape(g.ny, g.nx)
        else:
            v = vel.cpu().numpy()
            p = pres.cpu().numpy()
            velocity = v.T.copy() if two_d else v[0]
            pressure = np.moveaxis(p.reshape(-1, g.ny, g.nx), 0, -1).copy() if two_d else p[0].reshape(g.ny, g.nx)
        self.solve_seconds = self.solve_seconds  # already accumulated
        return StokesResult(velocity, pressure, float(info.residual), float(info.divergence_inf))
