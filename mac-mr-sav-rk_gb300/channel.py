"""Channel MAC flow (periodic x, stationary no-slip walls in y) on one GB300.

Mirrors the reference's ``solver/channel`` package: ``ChannelGrid``
(grid.py:9-104, host-side layout and validation), ``ChannelOperators``
(operators.py:9-25, here matrix-free device operators usable with ``@``),
``FFTStokes`` (fft_stokes.py:34-137, the banded per-mode saddle solves on the
GPU, see csrc/channel.cu) and ``ChannelModel`` (model.py:16-115, the model
seam with device vectors).  The reference's own scheme classes and drivers
run on ``ChannelModel`` unchanged (Level-2 drop-in).  ``backend='direct'``
maps to the same GPU FFT solver: the GPU has one channel Stokes solver, and
the reference tests the two backends to agree to 2e-12.
"""
from __future__ import annotations

import ctypes as C
from collections import OrderedDict
from collections.abc import Callable, Sequence
from dataclasses import dataclass
from time import perf_counter
from typing import Any

import numpy as np
import torch

from . import _lib
from .core import DeviceArray, Stage, State
from .stokes import StokesResult, dptr, stream_handle


@dataclass(frozen=True)
class ChannelGrid:
    """``solver/channel/grid.py:9-104``."""
    nx: int
    ny: int
    lx: float = 1.0
    ly: float = 1.0

    def __post_init__(self) -> None:
        if type(self.nx) is not int or type(self.ny) is not int or min(self.nx, self.ny) < 3:
            raise ValueError("Require integer nx,ny >= 3")
        if not np.isfinite([self.lx, self.ly]).all() or min(self.lx, self.ly) <= 0:
            raise ValueError("Require positive finite domain lengths")

    hx = property(lambda self: self.lx / self.nx)
    hy = property(lambda self: self.ly / self.ny)
    nu = property(lambda self: self.nx * self.ny)
    nv = property(lambda self: self.nx * (self.ny - 1))
    size = property(lambda self: self.nu + self.nv)
    np = property(lambda self: self.nx * self.ny)
    area = property(lambda self: self.hx * self.hy)

    def coordinates(self, field: str):
        if field == "u":
            x, y = np.arange(self.nx + 1) * self.hx, (np.arange(self.ny) + .5) * self.hy
        elif field == "v":
            x, y = (np.arange(self.nx) + .5) * self.hx, np.arange(self.ny + 1) * self.hy
        elif field == "p":
            x, y = (np.arange(self.nx) + .5) * self.hx, (np.arange(self.ny) + .5) * self.hy
        elif field == "vertex":
            x, y = np.arange(self.nx + 1) * self.hx, np.arange(self.ny + 1) * self.hy
        else:
            raise ValueError(f"Unknown field {field}")
        return np.meshgrid(x, y)

    def _faces(self, u, v) -> None:
        if u.shape != (self.ny, self.nx + 1) or v.shape != (self.ny + 1, self.nx):
            raise ValueError("Incorrect channel MAC array shapes")
        if np.iscomplexobj(u) or np.iscomplexobj(v) or not np.isfinite(u).all() or not np.isfinite(v).all():
            raise ValueError("Channel faces must be real and finite")
        tolerance = 32 * np.finfo(float).eps * max(1., float(np.max(np.abs(u))))
        if not np.allclose(u[:, 0], u[:, -1], rtol=0., atol=tolerance):
            raise ValueError("Streamwise u faces must be periodic")

    def pack(self, u, v) -> np.ndarray:
        self._faces(u, v)
        if np.any(v[[0, -1], :] != 0):
            raise ValueError("Normal wall velocities must be zero")
        return self.pack_load(u, v)

    def pack_load(self, u, v) -> np.ndarray:
        """Sample loads on free faces; a physical force at a wall need not vanish."""
        self._faces(u, v)
        return np.concatenate((u[:, :self.nx].ravel(), v[1:-1, :].ravel()))

    def unpack(self, velocity):
        velocity = np.asarray(velocity)
        if velocity.shape != (self.size,) or np.iscomplexobj(velocity) or not np.isfinite(velocity).all():
            raise ValueError("Incorrect or nonfinite channel free vector")
        u = np.empty((self.ny, self.nx + 1))
        u[:, :self.nx] = velocity[:self.nu].reshape(self.ny, self.nx)
        u[:, -1] = u[:, 0]
        v = np.zeros((self.ny + 1, self.nx))
        v[1:-1, :] = velocity[self.nu:].reshape(self.ny - 1, self.nx)
        return u, v

    def inner(self, a, b) -> float:
        return float(self.area * np.dot(np.asarray(a), np.asarray(b)))

    def norm(self, a) -> float:
        return float(np.sqrt(self.inner(a, a)))

    def curl(self, psi) -> np.ndarray:
        """Discrete vertex curl; each wall streamfunction must be constant in x."""
        if psi.shape != (self.ny + 1, self.nx + 1) or np.iscomplexobj(psi) or not np.isfinite(psi).all():
            raise ValueError("Incorrect or nonfinite vertex streamfunction")
        tolerance = 32 * np.finfo(float).eps * max(1., float(np.max(np.abs(psi))))
        if not np.allclose(psi[:, 0], psi[:, -1], rtol=0., atol=tolerance) \
                or np.max(np.ptp(psi[[0, -1], :], axis=1)) > tolerance:
            raise ValueError("Require periodic psi and constant wall psi")
        canonical = psi.copy()
        canonical[:, -1] = canonical[:, 0]
        canonical[0, :] = canonical[0, 0]
        canonical[-1, :] = canonical[-1, 0]
        return self.pack(np.diff(canonical, axis=0) / self.hy, -np.diff(canonical, axis=1) / self.hx)

    def metadata(self) -> dict[str, str]:
        return {"boundary": "periodic_x_no_slip_y", "discretization": "mac_second_order",
                "field_layout": "staggered_mac_periodic_x", "periodic_u_endpoint": "duplicated"}


class _Handle:
    """Owns one ``macsav_channel`` (the FFT solver's tables, factor cache and buffers)."""

    def __init__(self, grid: ChannelGrid, tolerance: float, cache_size: int) -> None:
        if not torch.cuda.is_available():
            raise RuntimeError("a CUDA device is required (the GB300 library has no CPU fallback)")
        self.lib = _lib.load()
        torch.cuda.init()
        h = C.c_void_p()
        code = self.lib.macsav_channel_create(C.byref(h), grid.nx, grid.ny, float(grid.lx), float(grid.ly),
                                              float(tolerance), int(cache_size))
        if code == _lib.ERR_UNSUPPORTED:
            raise ValueError("the GPU channel solver supports nx <= 2048")
        if code != _lib.OK:
            raise _lib.MacsavError(f"channel create failed (code {code})")
        self.handle = h

    def __del__(self) -> None:
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            self.lib.macsav_channel_destroy(h)
            self.handle = None

    def check(self, code: int) -> None:
        if code == _lib.OK:
            return
        msg = self.lib.macsav_channel_error(self.handle).decode()
        if code == _lib.ERR_VALUE:
            raise ValueError(msg)
        if code in (_lib.ERR_CG, _lib.ERR_STOKES_GATE):
            raise RuntimeError(msg)
        raise _lib.MacsavError(msg or f"macsav error code {code}")


def _dev(x) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        return x if (x.is_cuda and x.dtype == torch.float64) else x.to("cuda", torch.float64)
    if isinstance(x, DeviceArray):
        return x.tensor
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.float64))).to("cuda")


class _DeviceOperator:
    """Matrix-free channel operator: ``op @ x`` for NumPy (returns NumPy) or
    CUDA tensors (returns a tensor), vectors or column matrices."""

    def __init__(self, handle: _Handle, which: int, n_in: int, n_out: int) -> None:
        self.h, self.which, self.n_in, self.n_out = handle, which, n_in, n_out
        self.shape = (n_out, n_in)

    def __matmul__(self, x):
        is_torch = isinstance(x, torch.Tensor)
        t = _dev(x)
        two_d = t.ndim == 2
        cols = t.T.contiguous() if two_d else t.reshape(1, -1).contiguous()
        if cols.shape[1] != self.n_in:
            raise ValueError("operator shape mismatch")
        out = torch.empty((cols.shape[0], self.n_out), dtype=torch.float64, device="cuda")
        self.h.check(self.h.lib.macsav_channel_apply(self.h.handle, self.which, dptr(cols), dptr(out), cols.shape[0],
                                                     stream_handle()))
        res = out.T if two_d else out[0]
        return res if is_torch else res.cpu().numpy()


class ChannelOperators:
    """``solver/channel/operators.py:9-25`` as device operators ``K``, ``D``, ``G``."""

    def __init__(self, grid: ChannelGrid, handle: _Handle | None = None) -> None:
        self.grid = grid
        self.handle = handle if handle is not None else _Handle(grid, 1e-10, 1)
        self.K = _DeviceOperator(self.handle, 0, grid.size, grid.size)
        self.D = _DeviceOperator(self.handle, 1, grid.size, grid.np)
        self.G = _DeviceOperator(self.handle, 2, grid.np, grid.size)


class FFTStokes:
    """``solver/channel/fft_stokes.py:34-137`` on the GPU (csrc/channel.cu)."""

    def __init__(self, operators, cache_size: int = 4, tolerance: float = 1e-10) -> None:
        if type(cache_size) is not int or cache_size < 1 or not np.isfinite(tolerance) or tolerance <= 0:
            raise ValueError("Invalid channel FFT solver controls")
        self.ops = operators
        self.grid = operators.grid if hasattr(operators, "grid") else operators
        self.cache_size, self.tolerance = cache_size, tolerance
        self.handle = _Handle(self.grid, tolerance, cache_size)
        self.cache: OrderedDict[tuple[float, float], None] = OrderedDict()
        self.factorizations = 0
        self.factorization_seconds = 0.
        self.solve_seconds = 0.

    def solve_device(self, f: torch.Tensor, mass: float, viscosity: float):
        """Column-blocked device solve: f is (c, size) float64 CUDA."""
        g = self.grid
        c = f.shape[0]
        vel = torch.empty((c, g.size), dtype=torch.float64, device=f.device)
        pres = torch.empty((c, g.np), dtype=torch.float64, device=f.device)
        res, div, fact = C.c_double(), C.c_double(), C.c_int()
        start = perf_counter()
        code = self.handle.lib.macsav_channel_solve(self.handle.handle, dptr(f), c, float(mass), float(viscosity),
                                                    dptr(vel), dptr(pres), C.byref(res), C.byref(div),
                                                    C.byref(fact), stream_handle())
        elapsed = perf_counter() - start
        key = (float(mass), float(viscosity))
        if fact.value:
            self.factorizations += 1
            self.factorization_seconds += elapsed
            self.cache[key] = None
            if len(self.cache) > self.cache_size:
                self.cache.popitem(last=False)
        else:
            self.solve_seconds += elapsed
        if key in self.cache:
            self.cache.move_to_end(key)
        self.handle.check(code)
        return vel, pres, float(res.value), float(div.value)

    def solve(self, rhs, *, mass: float, viscosity: float) -> StokesResult:
        g = self.grid
        if not np.isfinite([mass, viscosity]).all() or min(mass, viscosity) < 0 or mass + viscosity <= 0:
            raise ValueError("Require nonnegative mass/viscosity with nonzero total")
        is_torch = isinstance(rhs, torch.Tensor)
        arr = rhs if is_torch else np.asarray(rhs)
        if arr.ndim not in (1, 2) or arr.shape[0] != g.size or (not is_torch and np.iscomplexobj(arr)) \
                or (is_torch and arr.is_complex()):
            raise ValueError("Invalid channel FFT RHS")
        if not is_torch and not np.isfinite(arr).all():
            raise ValueError("Invalid channel FFT RHS")
        two_d = arr.ndim == 2
        f = _dev(arr)
        if is_torch and not bool(torch.isfinite(f).all()):
            raise ValueError("Invalid channel FFT RHS")
        f = (f.T if two_d else f[None, :]).contiguous()
        vel, pres, res, div = self.solve_device(f, mass, viscosity)
        if is_torch:
            velocity = vel.T if two_d else vel[0]
            pressure = pres.reshape(-1, g.ny, g.nx).permute(1, 2, 0) if two_d else pres[0].reshape(g.ny, g.nx)
        else:
            v, p = vel.cpu().numpy(), pres.cpu().numpy()
            velocity = v.T.copy() if two_d else v[0]
            pressure = np.moveaxis(p.reshape(-1, g.ny, g.nx), 0, -1).copy() if two_d else p[0].reshape(g.ny, g.nx)
        return StokesResult(velocity, pressure, res, div)


def _zero_force(grid: ChannelGrid):
    def force(t: float) -> np.ndarray:
        return np.zeros(grid.size)
    force.zero = True
    return force


class ChannelModel:
    """``solver/channel/model.py:16-115`` with device vectors."""

    def __init__(self, grid: ChannelGrid, nu: float, force: Callable[[float], Any] | None = None,
                 backend: Any = None, cache_size: int = 4, tolerance: float = 1e-10) -> None:
        if not np.isfinite(nu) or nu <= 0:
            raise ValueError("nu must be positive and finite")
        self.grid, self.nu = grid, nu
        if backend is None or backend in ("direct", "fft"):
            self.backend = FFTStokes(grid, cache_size, tolerance)
        elif isinstance(backend, str):
            raise ValueError("Unknown channel backend")
        else:
            self.backend = backend
        handle = getattr(self.backend, "handle", None)
        self._h = handle if isinstance(handle, _Handle) else _Handle(grid, tolerance, cache_size)
        self.ops = ChannelOperators(grid, self._h)
        self.force = force if force is not None else _zero_force(grid)

    # --------------------------------------------------------------- plumbing
    def _apply(self, which: int, x, n_out: int) -> torch.Tensor:
        xd = _dev(x).reshape(1, -1).contiguous()
        out = torch.empty((1, n_out), dtype=torch.float64, device="cuda")
        self._h.check(self._h.lib.macsav_channel_apply(self._h.handle, which, dptr(xd), dptr(out), 1,
                                                       stream_handle()))
        return out[0]

    def _reduce(self, a, b=None) -> tuple[float, float]:
        ad = _dev(a).contiguous().reshape(-1)
        bd = _dev(b).contiguous().reshape(-1) if b is not None else None
        res = (C.c_double * 2)()
        self._h.check(self._h.lib.macsav_channel_reduce(self._h.handle, dptr(ad), dptr(bd) if bd is not None else None,
                                                        ad.numel(), res, stream_handle()))
        return float(res[0]), float(res[1])

    def device_vector(self, state: State) -> torch.Tensor:
        cached = getattr(state, "device", None)
        return cached if cached is not None else _dev(self.vector(state))

    # ------------------------------------------------------------------ seam
    def vector(self, state: State) -> np.ndarray:
        return self.grid.pack(state.u, state.v)

    def state(self, t: float, velocity, r: float = 0.) -> State:
        dv = _dev(velocity).contiguous()
        u, v = self.grid.unpack(dv.cpu().numpy())
        return State(t, u, v, float(r), dv)

    def nonlinear(self, velocity) -> torch.Tensor:
        return self._apply(3, velocity, self.grid.size)

    def nonlinear_with_lifting(self, velocity) -> tuple[torch.Tensor, float]:
        return self.nonlinear(velocity), 0.

    def combine(self, *terms) -> torch.Tensor:
        fields = [_dev(f).contiguous() for _, f in terms]
        out = torch.empty_like(fields[0])
        n = fields[0].numel()
        k = 0
        while k < len(terms) or k == 0:
            # the kernel takes 8 terms; later chunks add to the running sum in order
            take = 8 if k == 0 else 7
            idx = list(range(k, min(k + take, len(terms))))
            coeffs = ([] if k == 0 else [1.0]) + [float(terms[i][0]) for i in idx]
            ptrs = ([] if k == 0 else [out.data_ptr()]) + [fields[i].data_ptr() for i in idx]
            self._h.check(self._h.lib.macsav_channel_combine(
                self._h.handle, len(coeffs), (C.c_double * len(coeffs))(*coeffs),
                (C.c_void_p * len(ptrs))(*ptrs), dptr(out), n, stream_handle()))
            k += take
        return out

    def apply_K(self, velocity) -> torch.Tensor:
        return self._apply(0, velocity, self.grid.size)

    def apply_G(self, pressure) -> torch.Tensor:
        return self._apply(2, _dev(pressure).reshape(-1), self.grid.size)

    def apply_D(self, velocity) -> torch.Tensor:
        return self._apply(1, velocity, self.grid.np)

    def physical_divergence_inf(self, velocity) -> float:
        return self.max_abs(self.apply_D(velocity))

    def stage_divergences(self, velocity) -> tuple[float, float]:
        d = self.physical_divergence_inf(velocity)
        return d, d

    def inner(self, left, right) -> float:
        return self._reduce(left, right)[0]

    def max_abs(self, field) -> float:
        return self._reduce(field)[1]

    # Momentum adapter members (solver/momentum.py:36-52), so scheme code
    # written against the reference's stage_momentum runs on this model too.
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
        if isinstance(self.backend, FFTStokes):
            if not np.isfinite([mass, viscosity]).all() or min(mass, viscosity) < 0 or mass + viscosity <= 0:
                raise ValueError("Require nonnegative mass/viscosity with nonzero total")
            f = _dev(rhs).reshape(1, -1).contiguous()
            if f.shape[1] != self.grid.size or not bool(torch.isfinite(f).all()):
                raise ValueError("Invalid channel FFT RHS")
            vel, pres, res, div = self.backend.solve_device(f, mass, viscosity)
            return StokesResult(vel[0], pres[0].reshape(self.grid.ny, self.grid.nx), res, div)
        return self.backend.solve(rhs, mass=mass, viscosity=viscosity)

    def solve_columns(self, columns: Sequence[Any], *, mass: float, viscosity: float) -> list[StokesResult]:
        g = self.grid
        if isinstance(self.backend, FFTStokes):
            if not np.isfinite([mass, viscosity]).all() or min(mass, viscosity) < 0 or mass + viscosity <= 0:
                raise ValueError("Require nonnegative mass/viscosity with nonzero total")
            f = torch.stack([_dev(c).reshape(-1) for c in columns]).contiguous()
            if f.shape[1] != g.size or not bool(torch.isfinite(f).all()):
                raise ValueError("Invalid channel FFT RHS")
            vel, pres, res, div = self.backend.solve_device(f, mass, viscosity)
            return [StokesResult(vel[k], pres[k].reshape(g.ny, g.nx), res, div) for k in range(len(columns))]
        solved = self.solve(np.column_stack([np.asarray(c) for c in columns]), mass=mass, viscosity=viscosity)
        return [StokesResult(solved.velocity[:, k], solved.pressure[:, :, k], solved.residual, solved.divergence_inf)
                for k in range(len(columns))]

    def stage(self, pressure, residual: float, divergence_inf: float, r: float = 0.,
              candidates: Sequence[float] = (), root_residuals: Sequence[float] = (),
              scalar_residual: float = 0., *, continuity_residual: float = float("nan")) -> Stage:
        p = DeviceArray(pressure) if isinstance(pressure, torch.Tensor) else pressure
        return Stage(p, residual, divergence_inf, r, list(candidates), list(root_residuals), scalar_residual,
                     continuity_residual)

    def collocated_velocity(self, velocity):
        u, v = self.grid.unpack(_dev(velocity).cpu().numpy())
        return .5 * (u[:, :-1] + u[:, 1:]), .5 * (v[:-1] + v[1:])

    def flow_rates(self, velocity) -> np.ndarray:
        out = torch.empty(self.grid.nx, dtype=torch.float64, device="cuda")
        x = _dev(velocity).contiguous()
        self._h.check(self._h.lib.macsav_channel_flow_rates(self._h.handle, dptr(x), dptr(out), stream_handle()))
        return out.cpu().numpy()

    def diagnostics(self, state: State) -> dict[str, float]:
        """``model.py:98-115``, with the reductions on the device."""
        g = self.grid
        w = self.device_vector(state)
        kinetic = .5 * self.inner(w, w)
        h1 = self.inner(w, self.apply_K(w))
        flux = self.flow_rates(w)
        walls = w[:g.nx].cpu().numpy(), w[(g.ny - 1) * g.nx:g.ny * g.nx].cpu().numpy()
        force = self.force(state.t)
        return {"kinetic": kinetic, "modified_energy": kinetic + .5 * (state.r - 1) ** 2,
                "divergence_inf": self.physical_divergence_inf(w), "r": state.r,
                "h1_seminorm_squared": h1, "power": self.inner(force, w),
                "dissipation": self.nu * h1, "bulk_velocity": float(np.mean(flux) / g.ly),
                "flow_rate": float(np.mean(flux)), "flow_rate_spread": float(np.ptp(flux)),
                "wall_shear_bottom": float(2 * self.nu * np.mean(walls[0]) / g.hy),
                "wall_shear_top": float(-2 * self.nu * np.mean(walls[1]) / g.hy)}
