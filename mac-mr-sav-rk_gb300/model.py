"""GPU ``MACNavierStokes``: the reference's MAC model seam on the CUDA library.

Mirrors ``solver/mac_ns.py:12-107`` member for member.  Packed velocities and
pressures are float64 CUDA tensors; every operator (K, D, D^T, convection,
combine, inner, max_abs, diagnostics) runs in ``libmacsav.so`` through the C
ABI.  ``vector(state)`` returns the host packed array (the drivers call
``np.isfinite`` on it) and ``state(t, velocity, r)`` builds a host ``State``
that also carries the device copy.
"""
from __future__ import annotations

import ctypes as C
import warnings
from collections.abc import Callable, Sequence
from typing import Any

import numpy as np
import torch

from . import _lib
from .core import DeviceArray, Stage, State
from .grid import MACGrid
from .stokes import StokesResult, TensorStokes, dptr, stream_handle


def _zero_force(grid: MACGrid) -> Callable[[float], np.ndarray]:
    def force(t: float) -> np.ndarray:
        return np.zeros(grid.size)
    force.zero = True  # marks the default (no body force)
    return force


class MACNavierStokes:
    """No-slip MAC model (``solver/mac_ns.py:12-107``) on one GB300."""

    def __init__(self, grid: MACGrid, nu: float, force: Callable[[float], Any] | None = None,
                 backend: TensorStokes | None = None, cache_size: int = 4, *, precision: str = "fp64",
                 krylov_tolerance: float = 1e-12, tolerance: float = 1e-9, use_graph: bool = False,
                 corrections: int | None = None, inner_krylov_tolerance: float | None = None,
                 first_krylov_tolerance: float | None = None) -> None:
        if not np.isfinite(nu) or nu <= 0:
            raise ValueError("nu must be positive and finite")
        self.grid = grid
        self.nu = nu
        self.backend = backend if backend is not None else TensorStokes(
            grid, tolerance=tolerance, krylov_tolerance=krylov_tolerance, precision=precision,
            corrections=corrections, inner_krylov_tolerance=inner_krylov_tolerance,
            first_krylov_tolerance=first_krylov_tolerance)
        self.force = force if force is not None else _zero_force(grid)
        self.use_graph = use_graph
        self.device = torch.device("cuda")

    # ----------------------------------------------------------- plumbing ---
    @property
    def plan(self):
        return self.backend.plan

    def _dev(self, x) -> torch.Tensor:
        if isinstance(x, torch.Tensor):
            return x if (x.is_cuda and x.dtype == torch.float64) else x.to(self.device, torch.float64)
        if isinstance(x, DeviceArray):
            return x.tensor
        return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64))).to(self.device)

    def _op(self, name: str, x, out_len: int) -> torch.Tensor:
        xd = self._dev(x).contiguous()
        out = torch.empty(out_len, dtype=torch.float64, device=self.device)
        self.plan.check(getattr(self.plan.lib, name)(self.plan.handle, dptr(xd), dptr(out), 1, stream_handle()))
        return out

    def zero_velocity(self) -> torch.Tensor:
        return torch.zeros(self.grid.size, dtype=torch.float64, device=self.device)

    # --------------------------------------------------------------- seam ---
    def nonlinear(self, velocity) -> torch.Tensor:
        """Convection N(u) (mac_ns.py:22-25, kernels.py:6-35)."""
        return self._op("macsav_convection", velocity, self.grid.size)

    def nonlinear_with_lifting(self, velocity) -> tuple[torch.Tensor, float]:
        return self.nonlinear(velocity), 0.0

    def vector(self, state: State) -> np.ndarray:
        return self.grid.pack(state.u, state.v)

    def device_vector(self, state: State) -> torch.Tensor:
        """Packed device velocity of a state (its cached copy when it has one).
        A host state crosses as its two face arrays, packed on the device
        (after the wall-face check of MACGrid.pack, solver/mac/grid.py:52-57)."""
        cached = getattr(state, "device", None)
        if cached is not None:
            return cached
        g = self.grid
        u, v = np.asarray(state.u, dtype=np.float64), np.asarray(state.v, dtype=np.float64)
        if u.shape != (g.ny, g.nx + 1) or v.shape != (g.ny + 1, g.nx):
            raise ValueError("Incorrect MAC array shapes")
        if np.any(u[:, [0, -1]] != 0) or np.any(v[[0, -1], :] != 0):
            raise ValueError("Normal boundary velocities must be zero")
        if not (u.flags.writeable or v.flags.writeable) and self._host_mapped(u) and self._host_mapped(v):
            # read-only pinned face arrays (those of a State this model built):
            # the pack kernel reads them over the host link, no staging copy or
            # sync.  Writable arrays take the blocking copy, so a caller may
            # overwrite them as soon as this returns, as after MACGrid.pack.
            x = torch.empty(g.size, dtype=torch.float64, device=self.device)
            self.plan.check(self.plan.lib.macsav_layout(self.plan.handle, 1, dptr(x), u.ctypes.data, v.ctypes.data,
                                                        stream_handle()))
            x._host_faces = (u, v)  # keeps the pinned blocks alive while the kernel may read them
            return x
        with warnings.catch_warnings():
            # States hold read-only arrays; these host views are only read (copied to the device)
            warnings.filterwarnings("ignore", message="The given NumPy array is not writable")
            ud = torch.from_numpy(np.ascontiguousarray(u)).to(self.device)
            vd = torch.from_numpy(np.ascontiguousarray(v)).to(self.device)
        x = torch.empty(g.size, dtype=torch.float64, device=self.device)
        self.plan.check(self.plan.lib.macsav_layout(self.plan.handle, 1, dptr(x), dptr(ud), dptr(vd),
                                                    stream_handle()))
        return x

    def _mapped_range(self, ptr: int, nbytes: int) -> bool:
        ok = C.c_int()
        self.plan.check(self.plan.lib.macsav_host_mapped(ptr, nbytes, C.byref(ok)))
        return bool(ok.value)

    def _host_mapped(self, a: np.ndarray) -> bool:
        """True when host array ``a`` lies inside one pinned torch storage (its
        numpy base) that the device maps at the same address, so the layout
        kernels may read it directly; pageable and foreign arrays take the
        copy path."""
        base = a.base
        if not (isinstance(base, torch.Tensor) and a.flags.c_contiguous and a.dtype == np.float64
                and base.device.type == "cpu" and base.is_pinned()):
            return False
        st = base.untyped_storage()
        lo, p = st.data_ptr(), a.ctypes.data
        if not (lo <= p and p + a.nbytes <= lo + st.nbytes()):
            return False
        return self._mapped_range(p, a.nbytes)

    def state(self, t: float, velocity, r: float = 0.0) -> State:
        """A host State (face arrays unpacked on the device) that also keeps
        the packed device vector.  The host arrays live in pinned memory from
        torch's caching host allocator, which the device maps: the unpack
        kernel writes them over the host link (NVLink-C2C on a Grace host)
        and a later ``device_vector`` of the same arrays packs from them
        directly, with no staging copies; the blocks of dropped states are
        reused instead of faulting in fresh pages (on the Grace host a GPU
        write into fresh pageable pages of this size cost about 2.5 ms).
        Where the pinned blocks are not mapped, the arrays are copied."""
        dv = self._dev(velocity).contiguous()
        g = self.grid
        if dv.numel() != g.size:
            raise ValueError("Incorrect free-vector shape")
        hu = torch.empty((g.ny, g.nx + 1), dtype=torch.float64, pin_memory=True)
        hv = torch.empty((g.ny + 1, g.nx), dtype=torch.float64, pin_memory=True)
        if self._mapped_range(hu.data_ptr(), hu.nbytes) and self._mapped_range(hv.data_ptr(), hv.nbytes):
            # the unpack kernel writes the pinned host arrays over the host link
            self.plan.check(self.plan.lib.macsav_layout(self.plan.handle, 0, dptr(dv), hu.data_ptr(), hv.data_ptr(),
                                                        stream_handle()))
        else:
            ud = torch.empty(hu.shape, dtype=torch.float64, device=self.device)
            vd = torch.empty(hv.shape, dtype=torch.float64, device=self.device)
            self.plan.check(self.plan.lib.macsav_layout(self.plan.handle, 0, dptr(dv), dptr(ud), dptr(vd),
                                                        stream_handle()))
            hu.copy_(ud, non_blocking=True)
            hv.copy_(vd, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        u, v = hu.numpy(), hv.numpy()
        u.flags.writeable = False
        v.flags.writeable = False
        return State(t, u, v, float(r), dv)

    def combine(self, *terms: tuple[float, Any]) -> torch.Tensor:
        """Sum of coefficient*field pairs in the given order (mac_ns.py:40-45)."""
        fields = [self._dev(f).contiguous() for _, f in terms]
        n = fields[0].numel()
        out = torch.empty_like(fields[0])
        coeffs = (C.c_double * len(terms))(*[float(c) for c, _ in terms])
        ptrs = (C.c_void_p * len(terms))(*[f.data_ptr() for f in fields])
        self.plan.check(self.plan.lib.macsav_combine(self.plan.handle, len(terms), coeffs, ptrs, dptr(out), n,
                                                     stream_handle()))
        return out

    def apply_K(self, velocity) -> torch.Tensor:
        return self._op("macsav_apply_K", velocity, self.grid.size)

    def apply_G(self, pressure) -> torch.Tensor:
        """G = -D^T (operators.py:30, mac_ns.py:50-51)."""
        return -self._op("macsav_apply_Dt", self._dev(pressure).reshape(-1), self.grid.size)

    def apply_D(self, velocity) -> torch.Tensor:
        return self._op("macsav_apply_D", velocity, self.grid.np)

    def physical_divergence_inf(self, velocity) -> float:
        return self.max_abs(self.apply_D(velocity))

    def stage_divergences(self, velocity) -> tuple[float, float]:
        d = self.max_abs(self.apply_D(velocity))
        return d, d

    def inner(self, left, right) -> float:
        a, b = self._dev(left).contiguous(), self._dev(right).contiguous()
        res = C.c_double()
        self.plan.check(self.plan.lib.macsav_inner(self.plan.handle, dptr(a), dptr(b), a.numel(), C.byref(res),
                                                   stream_handle()))
        return float(res.value)

    def max_abs(self, field) -> float:
        a = self._dev(field).contiguous().reshape(-1)
        res = C.c_double()
        self.plan.check(self.plan.lib.macsav_max_abs(self.plan.handle, dptr(a), a.numel(), C.byref(res),
                                                     stream_handle()))
        return float(res.value)

    # Momentum adapter members (solver/momentum.py:36-52), so scheme code written
    # against the reference's stage_momentum runs on this model too.
    def pair(self, load, velocity) -> float:
        return self.inner(load, velocity)

    def cauchy_scale(self, load, velocity) -> float:
        return float(np.sqrt(self.inner(load, load) * self.inner(velocity, velocity)))

    def residual(self, defect, rhs, convection=None, factor: float = 0.0) -> float:
        denominator = 1 + self.max_abs(rhs)
        if convection is not None:
            denominator += factor * self.max_abs(convection)
        return self.max_abs(defect) / denominator

    def solve(self, rhs, *, mass: float, viscosity: float) -> StokesResult:
        f = self._dev(rhs).reshape(1, -1).contiguous()
        vel, pres, info = self.backend.solve_device(f, mass, viscosity)
        g = self.grid
        return StokesResult(vel[0], pres[0].reshape(g.ny, g.nx), float(info.residual), float(info.divergence_inf))

    def solve_columns(self, columns: Sequence[Any], *, mass: float, viscosity: float) -> list[StokesResult]:
        """One batched solve split into per-column results (mac_ns.py:72-77)."""
        f = torch.stack([self._dev(c).reshape(-1) for c in columns]).contiguous()
        vel, pres, info = self.backend.solve_device(f, mass, viscosity)
        g = self.grid
        return [StokesResult(vel[k], pres[k].reshape(g.ny, g.nx), float(info.residual), float(info.divergence_inf))
                for k in range(len(columns))]

    def stage(self, pressure, residual: float, divergence_inf: float, r: float = 0.,
              candidates: Sequence[float] = (), root_residuals: Sequence[float] = (),
              scalar_residual: float = 0., *, continuity_residual: float = float("nan")) -> Stage:
        p = pressure if isinstance(pressure, DeviceArray) else (
            DeviceArray(pressure) if isinstance(pressure, torch.Tensor) else pressure)
        return Stage(p, residual, divergence_inf, r, list(candidates), list(root_residuals), scalar_residual,
                     continuity_residual)

    def collocated_velocity(self, velocity) -> tuple[np.ndarray, np.ndarray]:
        u, v = self.grid.unpack(np.asarray(self._dev(velocity).cpu().numpy()))
        return 0.5 * (u[:, :-1] + u[:, 1:]), 0.5 * (v[:-1, :] + v[1:, :])

    def angular_momentum(self, velocity) -> float:
        return self._diagnostics(self._dev(velocity), 0.0, None)[5]

    def _force_device(self, t: float):
        if getattr(self.force, "zero", False):
            return None
        return self._dev(self.force(t)).contiguous()

    def _diagnostics(self, x: torch.Tensor, r: float, force) -> list[float]:
        out = (C.c_double * 8)()
        x = x.contiguous()
        self.plan.check(self.plan.lib.macsav_diagnostics(self.plan.handle, dptr(x), float(r), float(self.nu),
                                                         dptr(force) if force is not None else None, out,
                                                         stream_handle()))
        return list(out)

    def diagnostics(self, state: State) -> dict[str, float]:
        """kinetic, modified energy, divergence, H1, r, angular momentum, power,
        dissipation (mac_ns.py:95-107), reduced on the device."""
        d = self._diagnostics(self.device_vector(state), state.r, self._force_device(state.t))
        keys = ("kinetic", "modified_energy", "divergence_inf", "h1_seminorm_squared", "r", "angular_momentum",
                "power", "dissipation")
        return dict(zip(keys, (float(v) for v in d)))
