"""NumPy/SciPy restatement of the reference's MAC mr-SAV hot path (test oracle).

Every function names the reference file:line whose behaviour it restates
(paths are relative to the HaifengWang1031/MAC-mr-SAV-RK project root).  The
pinned third-party arithmetic is the reference's own: SciPy 1.18.1
``scipy.fft.dst/dct`` with ``norm="ortho"`` and ``scipy.sparse.linalg.cg``
(``uv.lock:973-974``).  Numba (``uv.lock:641-642``) only JIT-compiles loops in
the reference; the loops are restated here as vectorised NumPy.

Nothing here runs on a GPU; it is the CPU checker only.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from time import perf_counter
from typing import Any, Callable, Sequence

import numpy as np
from scipy.fft import dct, dst, idct, idst
from scipy.sparse.linalg import LinearOperator, cg

__all__ = [
    "Grid", "apply_K", "apply_D", "apply_Dt", "convection", "nonlinear",
    "eigenvalues_1d", "trig_transform", "StokesResult", "TensorStokesOracle",
    "solve_scalar_stage", "ScalarCorrection", "State", "Stage", "Trial",
    "OracleModel", "SDIRK2MRSAV", "SDIRK3MRSAV", "SDIRK2", "SDIRK3",
    "IMEXEuler", "IMEXEulerMRSAV", "make_scheme", "integrate", "Result",
    "ETA", "DELTA", "D3", "DHAT3", "C3", "schedule_nodes", "nearest_node_indices",
    "stage_diagnostics",
]


# --------------------------------------------------------------------------- grid
@dataclass(frozen=True)
class Grid:
    """Uniform staggered layout (``solver/mac/grid.py:9-71``).

    u is (ny, nx+1), v is (ny+1, nx), p is (ny, nx); axis 0 is y.  The packed
    free vector is [u[:,1:-1].ravel(), v[1:-1,:].ravel()] (grid.py:52-57).
    """
    nx: int
    ny: int
    lx: float = 1.0
    ly: float = 1.0

    def __post_init__(self) -> None:  # grid.py:15-19
        if min(self.nx, self.ny) < 3 or min(self.lx, self.ly) <= 0:
            raise ValueError("Require nx,ny >= 3 and positive finite domain lengths")

    hx = property(lambda s: s.lx / s.nx)
    hy = property(lambda s: s.ly / s.ny)
    n_u = property(lambda s: (s.nx - 1) * s.ny)
    n_v = property(lambda s: s.nx * (s.ny - 1))
    size = property(lambda s: s.n_u + s.n_v)
    np = property(lambda s: s.nx * s.ny)
    area = property(lambda s: s.hx * s.hy)

    def coordinates(self, kind: str) -> tuple[np.ndarray, np.ndarray]:
        """Face/cell/vertex coordinates (grid.py:36-50)."""
        hx, hy, nx, ny = self.hx, self.hy, self.nx, self.ny
        xs = {"u": np.arange(nx + 1) * hx, "v": (np.arange(nx) + .5) * hx,
              "p": (np.arange(nx) + .5) * hx, "vertex": np.arange(nx + 1) * hx}[kind]
        ys = {"u": (np.arange(ny) + .5) * hy, "v": np.arange(ny + 1) * hy,
              "p": (np.arange(ny) + .5) * hy, "vertex": np.arange(ny + 1) * hy}[kind]
        return np.meshgrid(xs.astype(float), ys.astype(float))

    def pack(self, u: np.ndarray, v: np.ndarray) -> np.ndarray:  # grid.py:52-57
        if u.shape != (self.ny, self.nx + 1) or v.shape != (self.ny + 1, self.nx):
            raise ValueError("Incorrect MAC array shapes")
        if np.any(u[:, [0, -1]] != 0) or np.any(v[[0, -1], :] != 0):
            raise ValueError("Normal boundary velocities must be zero")
        return np.concatenate((u[:, 1:-1].ravel(), v[1:-1, :].ravel()))

    def unpack(self, x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:  # grid.py:59-65
        if x.shape != (self.size,):
            raise ValueError("Incorrect free-vector shape")
        u = np.zeros((self.ny, self.nx + 1))
        v = np.zeros((self.ny + 1, self.nx))
        u[:, 1:-1] = x[:self.n_u].reshape(self.ny, self.nx - 1)
        v[1:-1, :] = x[self.n_u:].reshape(self.ny - 1, self.nx)
        return u, v

    def inner(self, a: np.ndarray, b: np.ndarray) -> float:  # grid.py:67-68
        return float(self.area * np.dot(a, b))

    def norm(self, a: np.ndarray) -> float:  # grid.py:70-71
        return float(np.sqrt(self.inner(a, a)))


# ---------------------------------------------------------------------- stencils
def _lap1d(a: np.ndarray, axis: int, h: float, wall: bool) -> np.ndarray:
    """Positive 1-D second difference along ``axis`` with zero Dirichlet ghosts.

    ``wall=True`` is the tangential half-cell wall of ``operators.py:6-9``:
    the end diagonal is 3/h^2 instead of 2/h^2.
    """
    a = np.moveaxis(a, axis, 0)
    out = 2.0 * a
    out[1:] -= a[:-1]
    out[:-1] -= a[1:]
    if wall:
        out[0] += a[0]
        out[-1] += a[-1]
    return np.moveaxis(out / (h * h), 0, axis)


def apply_K(g: Grid, x: np.ndarray) -> np.ndarray:
    """K = blockdiag(Ku, Kv) of ``solver/mac/operators.py:16-18`` (matrix free).

    Ku = I_y (x) L_x(nx-1, plain) + L_y(ny, wall) (x) I_x;
    Kv = I_y (x) L_x(nx, wall) + L_y(ny-1, plain) (x) I_x.
    """
    u = x[:g.n_u].reshape(g.ny, g.nx - 1, -1)
    v = x[g.n_u:].reshape(g.ny - 1, g.nx, -1)
    ku = _lap1d(u, 1, g.hx, False) + _lap1d(u, 0, g.hy, True)
    kv = _lap1d(v, 1, g.hx, True) + _lap1d(v, 0, g.hy, False)
    return np.concatenate((ku.reshape(g.n_u, -1), kv.reshape(g.n_v, -1))).reshape(x.shape)


def apply_D(g: Grid, x: np.ndarray) -> np.ndarray:
    """Packed cell divergence, walls eliminated (``operators.py:19-29``,
    ``kernels.py:46-87``).  Accepts (size,) or (size, c)."""
    cols = x.reshape(g.size, -1)
    out = np.zeros((g.ny, g.nx, cols.shape[1]))
    u = cols[:g.n_u].reshape(g.ny, g.nx - 1, -1) / g.hx
    v = cols[g.n_u:].reshape(g.ny - 1, g.nx, -1) / g.hy
    out[:, :-1] += u
    out[:, 1:] -= u
    out[:-1, :] += v
    out[1:, :] -= v
    return out.reshape(g.np) if x.ndim == 1 else out.reshape(g.np, -1)


def apply_Dt(g: Grid, p: np.ndarray) -> np.ndarray:
    """D^T p = -G p (``operators.py:30``, ``kernels.py:89-132``)."""
    cols = p.reshape(g.ny, g.nx, -1)
    u = (cols[:, :-1] - cols[:, 1:]) / g.hx
    v = (cols[:-1, :] - cols[1:, :]) / g.hy
    out = np.concatenate((u.reshape(g.n_u, -1), v.reshape(g.n_v, -1)))
    return out[:, 0] if p.ndim == 1 else out


def convection(u: np.ndarray, v: np.ndarray, hx: float, hy: float) -> tuple[np.ndarray, np.ndarray]:
    """Skew-symmetric centred dual-cell convection (``solver/mac/kernels.py:6-35``).

    Conservative flux form minus half the dual-cell divergence times the
    transported value; tangential ghosts across a wall are the odd reflection.
    """
    # u momentum at interior u faces (j, i), i = 1..nx-1
    uc = u[:, 1:-1]
    ue, uw = u[:, 2:], u[:, :-2]
    # odd ghosts: one row beyond each tangential wall
    ug = np.vstack((-u[:1], u, -u[-1:]))
    un, us = ug[2:, 1:-1], ug[:-2, 1:-1]
    fe, fw = .5 * (uc + ue), .5 * (uc + uw)
    fn, fs = .5 * (v[1:, :-1] + v[1:, 1:]), .5 * (v[:-1, :-1] + v[:-1, 1:])
    cu = (fe * fe - fw * fw) / hx + (fn * .5 * (uc + un) - fs * .5 * (uc + us)) / hy
    cu -= .5 * uc * ((fe - fw) / hx + (fn - fs) / hy)
    # v momentum at interior v faces (j, i), j = 1..ny-1
    vc = v[1:-1, :]
    vg = np.hstack((-v[:, :1], v, -v[:, -1:]))
    ve, vw = vg[1:-1, 2:], vg[1:-1, :-2]
    vn, vs = v[2:, :], v[:-2, :]
    ge, gw = .5 * (u[:-1, 1:] + u[1:, 1:]), .5 * (u[:-1, :-1] + u[1:, :-1])
    gn, gs = .5 * (vc + vn), .5 * (vc + vs)
    cv = (ge * .5 * (vc + ve) - gw * .5 * (vc + vw)) / hx + (gn * gn - gs * gs) / hy
    cv -= .5 * vc * ((ge - gw) / hx + (gn - gs) / hy)
    out_u = np.zeros_like(u)
    out_v = np.zeros_like(v)
    out_u[:, 1:-1] = cu
    out_v[1:-1, :] = cv
    return out_u, out_v


def nonlinear(g: Grid, x: np.ndarray) -> np.ndarray:
    """``MACNavierStokes.nonlinear`` (``solver/mac_ns.py:22-25``)."""
    u, v = g.unpack(x)
    cu, cv = convection(u, v, g.hx, g.hy)
    return g.pack(cu, cv)


# -------------------------------------------------------------------- transforms
def eigenvalues_1d(n: int, h: float, kind: str) -> np.ndarray:
    """Discrete 1-D eigenvalues (2-2cos theta)/h^2 (``tensor_stokes.py:31-38``)."""
    if kind == "dct2":
        theta = np.pi * np.arange(n) / n
    elif kind == "dst1":
        theta = np.pi * np.arange(1, n + 1) / (n + 1)
    elif kind == "dst2":
        theta = np.pi * np.arange(1, n + 1) / n
    else:
        raise ValueError(kind)
    return (2.0 - 2.0 * np.cos(theta)) / h ** 2


def trig_transform(a: np.ndarray, kind: str, axis: int, inverse: bool, workers: int = 1) -> np.ndarray:
    """Orthonormal DST-I / DST-II / DCT-II and inverses (``tensor_stokes.py:58-82``)."""
    if kind == "dct2":
        fn = idct if inverse else dct
        return fn(a, type=2, axis=axis, norm="ortho", workers=workers)
    fn = idst if inverse else dst
    return fn(a, type=1 if kind == "dst1" else 2, axis=axis, norm="ortho", workers=workers)


class _Basis:
    """Tensor eigenbasis of one block (``tensor_stokes.py:21-55``)."""

    def __init__(self, shape, spacing, kinds):
        (ny, nx), (hy, hx), (ky, kx) = shape, spacing, kinds
        self.kinds = (ky, kx)
        self.eig = eigenvalues_1d(ny, hy, ky)[:, None] + eigenvalues_1d(nx, hx, kx)[None, :]

    def forward(self, a, workers):  # tensor_stokes.py:85-101, axis 0 then axis 1
        return trig_transform(trig_transform(a, self.kinds[0], 0, False, workers), self.kinds[1], 1, False, workers)

    def inverse(self, a, workers):
        return trig_transform(trig_transform(a, self.kinds[0], 0, True, workers), self.kinds[1], 1, True, workers)


@dataclass
class StokesResult:
    """``solver/mac/stokes.py:32-37``."""
    velocity: np.ndarray
    pressure: np.ndarray
    residual: float
    divergence_inf: float


def _means(a: np.ndarray) -> np.ndarray:
    return a.mean(axis=0)


class TensorStokesOracle:
    """Restatement of ``TensorStokes`` (``solver/mac/tensor_stokes.py:118-364``).

    Velocity Helmholtz blocks are inverted by orthonormal tensor transforms:
    u by DST-II (y, len ny) x DST-I (x, len nx-1); v by DST-I (y, len ny-1) x
    DST-II (x, len nx); the pressure Poisson pseudo-inverse by DCT-II x DCT-II
    with the zero mode masked (:156-168).  The pressure Schur complement
    S = D (mI + kK)^-1 D^T is solved per column by SciPy's PCG with the
    preconditioner m (D D^T)^+ + k I (:272-325).
    """

    def __init__(self, grid: Grid, tolerance: float = 1e-9, krylov_tolerance: float = 1e-12,
                 max_iterations: int = 100, workers: int = 1) -> None:
        if (tolerance <= 0 or krylov_tolerance <= 0 or max_iterations < 1
                or not np.isfinite([tolerance, krylov_tolerance]).all()):
            raise ValueError("Invalid solver controls")  # tensor_stokes.py:137-143
        start = perf_counter()
        g = self.grid = grid
        self.tolerance, self.krylov_tolerance = tolerance, krylov_tolerance
        self.max_iterations, self.workers = max_iterations, workers
        self.u_basis = _Basis((g.ny, g.nx - 1), (g.hy, g.hx), ("dst2", "dst1"))
        self.v_basis = _Basis((g.ny - 1, g.nx), (g.hy, g.hx), ("dst1", "dst2"))
        self.p_basis = _Basis((g.ny, g.nx), (g.hy, g.hx), ("dct2", "dct2"))
        self.p_positive = self.p_basis.eig > 100.0 * np.finfo(float).eps * float(self.p_basis.eig.max())
        self.setup_seconds = perf_counter() - start
        self.solve_seconds = 0.0
        self.solves = self.right_hand_sides = self.total_iterations = 0
        self.last_iterations: tuple[int, ...] = ()

    # tensor_stokes.py:200-215
    def velocity_inverse(self, values: np.ndarray, mass: float, viscosity: float) -> np.ndarray:
        g = self.grid
        c = values.shape[1]
        out = []
        for basis, part, shape in ((self.u_basis, values[:g.n_u], (g.ny, g.nx - 1)),
                                   (self.v_basis, values[g.n_u:], (g.ny - 1, g.nx))):
            hat = basis.forward(part.reshape(*shape, c), self.workers)
            hat /= (mass + viscosity * basis.eig)[:, :, None]
            out.append(basis.inverse(hat, self.workers).reshape(-1, c))
        return np.vstack(out)

    # tensor_stokes.py:217-243
    def poisson_inverse(self, values: np.ndarray) -> np.ndarray:
        g = self.grid
        cols = values.reshape(g.np, -1)
        cols = cols - _means(cols)
        hat = self.p_basis.forward(cols.reshape(g.ny, g.nx, -1), self.workers)
        hat = np.divide(hat, self.p_basis.eig[:, :, None], out=np.zeros_like(hat),
                        where=self.p_positive[:, :, None])
        res = self.p_basis.inverse(hat, self.workers).reshape(g.np, -1)
        return res - _means(res)

    def solve(self, rhs: np.ndarray, *, mass: float, viscosity: float) -> StokesResult:
        """``TensorStokes.solve`` (tensor_stokes.py:245-364)."""
        g = self.grid
        if not np.isfinite([mass, viscosity]).all() or min(mass, viscosity) < 0 or mass + viscosity <= 0:
            raise ValueError("Require mass,viscosity >= 0 and nonzero total")
        if rhs.ndim not in (1, 2) or rhs.shape[0] != g.size or not np.isfinite(rhs).all():
            raise ValueError("Invalid Stokes RHS")
        start = perf_counter()
        two_d = rhs.ndim == 2
        force = np.asarray(rhs, dtype=float).reshape(g.size, -1)
        inv_force = self.velocity_inverse(force, mass, viscosity)
        p_rhs = -apply_D(g, inv_force)
        p_rhs = p_rhs - _means(p_rhs)

        def schur(p):  # :272-279
            p = p[:, None] - _means(p[:, None])
            res = apply_D(g, self.velocity_inverse(apply_Dt(g, p), mass, viscosity))
            return (res - _means(res))[:, 0]

        def precond(p):  # :281-287
            p = p[:, None] - _means(p[:, None])
            res = mass * self.poisson_inverse(p) + viscosity * p
            return (res - _means(res))[:, 0]

        n = g.np
        S = LinearOperator((n, n), matvec=schur, dtype=float)
        M = LinearOperator((n, n), matvec=precond, dtype=float)
        pressures = np.empty_like(p_rhs)
        counts = []
        for k in range(force.shape[1]):  # :302-325
            calls = [0]

            def cb(_):
                calls[0] += 1
            if np.max(np.abs(p_rhs[:, k])) == 0.0:
                pk, info = np.zeros(n), 0
            else:
                pk, info = cg(S, p_rhs[:, k], M=M, rtol=self.krylov_tolerance, atol=0.0,
                              maxiter=self.max_iterations, callback=cb)
            if info != 0:
                raise RuntimeError(f"Pressure Schur CG failed with info={info}")
            pressures[:, k] = pk - pk.mean()
            counts.append(calls[0])
        pressures -= _means(pressures)
        lift = apply_Dt(g, pressures)  # :329-331
        velocity = self.velocity_inverse(force + lift, mass, viscosity)
        defect = mass * velocity + viscosity * apply_K(g, velocity) - lift - force
        residual = float(np.max(np.abs(defect)) / (1 + np.max(np.abs(force))))
        divergence = float(np.max(np.abs(apply_D(g, velocity))))
        self.solve_seconds += perf_counter() - start
        self.solves += 1
        self.right_hand_sides += force.shape[1]
        self.total_iterations += sum(counts)
        self.last_iterations = tuple(counts)
        if (not np.isfinite(velocity).all() or not np.isfinite(pressures).all()
                or residual > self.tolerance
                or divergence > self.tolerance * (1 + np.max(np.abs(velocity)))):
            raise RuntimeError(f"Stokes residual={residual:.3e}, divergence={divergence:.3e}")
        if not two_d:
            return StokesResult(velocity[:, 0], pressures[:, 0].reshape(g.ny, g.nx), residual, divergence)
        return StokesResult(velocity, pressures.reshape(g.ny, g.nx, -1), residual, divergence)


# ------------------------------------------------------------ SAV scalar update
@dataclass(frozen=True)
class ScalarCorrection:
    """``solver/schemes/scalar_correction.py:9-27``."""
    predictor: float
    values: tuple
    factor: float

    @property
    def r(self) -> float:
        return self.values[-1]

    @property
    def coupling(self) -> float:
        return self.factor * (1 - self.r)

    def record(self, stage: "Stage") -> "Stage":
        stage.correction_predictor = self.predictor
        stage.corrections = list(self.values)
        stage.frozen_factor = self.factor
        return stage


def solve_scalar_stage(predictor: float, dt: float, d: float, rhs: float, alpha: float, beta: float,
                       *, order: int) -> ScalarCorrection:
    """Fixed-count frozen-factor map Phi (``scalar_correction.py:29-52``).

    Phi(z) = (R - dt C alpha + dt^2 C^2 beta) / (d + dt^2 C^2 beta) with
    C = P_{order-1}(z) in {1, 1+z, 1+z+z^2}; applied once for orders 1 and 2,
    twice for order 3.  The factor returned is C at the penultimate iterate.
    """
    if order not in (1, 2, 3):
        raise ValueError("SAV order must be 1, 2 or 3")
    if not np.isfinite([predictor, dt, d, rhs, alpha, beta]).all() or dt <= 0 or d <= 0 or beta < 0:
        raise ValueError("Invalid frozen SAV scalar inputs")
    z = predictor
    vals = []
    c = 1.0
    for _ in range(2 if order == 3 else 1):
        c = 1.0 if order == 1 else (1 + z if order == 2 else 1 + z + z * z)
        resp = dt * dt * c * c * beta
        den = d + resp
        if not np.isfinite(den) or den <= 0:
            raise RuntimeError("Invalid frozen SAV scalar denominator")
        z = (rhs - dt * c * alpha + resp) / den
        if not np.isfinite(z):
            raise RuntimeError("Nonfinite frozen SAV correction")
        vals.append(float(z))
    return ScalarCorrection(float(predictor), tuple(vals), float(c))


# ------------------------------------------------------------------ seam types
@dataclass(frozen=True)
class State:  # solver/core.py:8-12
    t: float
    u: np.ndarray
    v: np.ndarray
    r: float = 0.0


@dataclass
class Stage:  # solver/core.py:15-26
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


def stage_diagnostics(s: Stage) -> dict:  # solver/core.py:29-36
    return {"r": s.r, "candidates": s.candidates, "root_residuals": s.root_residuals,
            "root_count": len(s.candidates), "residual": s.residual,
            "scalar_residual": s.scalar_residual, "divergence_inf": s.divergence_inf,
            "continuity_residual": s.continuity_residual,
            "correction_predictor": s.correction_predictor, "corrections": s.corrections,
            "correction_count": len(s.corrections), "frozen_factor": s.frozen_factor}


@dataclass
class Trial:  # solver/core.py:39-42
    state: State
    stages: list
    embedded_velocity: Any = None


class OracleModel:
    """The MAC model seam (``solver/mac_ns.py:12-107``) over the oracle kernels."""

    def __init__(self, grid: Grid, nu: float, force: Callable | None = None, backend=None) -> None:
        if not np.isfinite(nu) or nu <= 0:
            raise ValueError("nu must be positive and finite")
        self.grid, self.nu = grid, nu
        self.backend = backend if backend is not None else TensorStokesOracle(grid)
        self.force = force if force is not None else (lambda t: np.zeros(grid.size))

    def nonlinear(self, x):
        return nonlinear(self.grid, x)

    def nonlinear_with_lifting(self, x):
        return self.nonlinear(x), 0.0

    def vector(self, s: State):
        return self.grid.pack(s.u, s.v)

    def state(self, t, x, r=0.0):
        u, v = self.grid.unpack(x)
        return State(t, u, v, r)

    def combine(self, *terms):  # mac_ns.py:40-45, summed in the order given
        total = np.zeros_like(terms[0][1], dtype=float)
        for c, f in terms:
            total += c * f
        return total

    def apply_K(self, x):
        return apply_K(self.grid, x)

    def apply_G(self, p):
        return -apply_Dt(self.grid, np.asarray(p).reshape(-1))

    def apply_D(self, x):
        return apply_D(self.grid, x)

    def stage_divergences(self, x):  # mac_ns.py:59-61
        d = self.max_abs(self.apply_D(x))
        return d, d

    def inner(self, a, b):
        return self.grid.inner(a, b)

    def max_abs(self, f):
        return float(np.max(np.abs(f)))

    def pair(self, a, b):  # solver/momentum.py:36-37
        return self.inner(a, b)

    def cauchy_scale(self, a, b):  # momentum.py:39-40
        return float(np.sqrt(self.inner(a, a) * self.inner(b, b)))

    def residual(self, defect, rhs, conv=None, factor=0.0):  # momentum.py:48-52
        den = 1 + self.max_abs(rhs)
        if conv is not None:
            den += factor * self.max_abs(conv)
        return self.max_abs(defect) / den

    def solve(self, rhs, *, mass, viscosity):
        return self.backend.solve(rhs, mass=mass, viscosity=viscosity)

    def solve_columns(self, cols, *, mass, viscosity):  # mac_ns.py:72-77
        out = self.backend.solve(np.column_stack(cols), mass=mass, viscosity=viscosity)
        return [StokesResult(out.velocity[:, k], out.pressure[:, :, k], out.residual, out.divergence_inf)
                for k in range(len(cols))]

    def stage(self, pressure, residual, divergence_inf, r=0.0, scalar_residual=0.0, *,
              continuity_residual=float("nan")):
        return Stage(pressure, residual, divergence_inf, r, [], [], scalar_residual, continuity_residual)

    def angular_momentum(self, x):  # mac_ns.py:84-93
        g = self.grid
        u, v = g.unpack(x)
        cu, cv = .5 * (u[:, :-1] + u[:, 1:]), .5 * (v[:-1, :] + v[1:, :])
        xs, ys = g.coordinates("p")
        return float(g.area * np.sum((xs - .5 * g.lx) * cv - (ys - .5 * g.ly) * cu))

    def diagnostics(self, s: State) -> dict:  # mac_ns.py:95-107
        g = self.grid
        x = self.vector(s)
        kinetic = .5 * g.inner(x, x)
        h1 = g.inner(x, apply_K(g, x))
        return {"kinetic": kinetic, "modified_energy": kinetic + .5 * (s.r - 1) ** 2,
                "divergence_inf": float(np.max(np.abs(apply_D(g, x)))),
                "h1_seminorm_squared": h1, "r": s.r, "angular_momentum": self.angular_momentum(x),
                "power": g.inner(self.force(s.t), x), "dissipation": self.nu * h1}


# -------------------------------------------------------------------- schemes
ETA = 1 - 1 / np.sqrt(2.0)  # solver/schemes/sdirk2.py:14
DELTA = -1 / np.sqrt(2.0)   # sdirk2.py:15
D3 = np.array([[1 / 4, 0, 0, 0], [3 / 10, 1 / 4, 0, 0],          # sdirk3.py:8-9
               [-31 / 220, 1 / 11, 1 / 4, 0], [31 / 198, 5 / 132, -4 / 9, 1 / 4]])
DHAT3 = np.array([[1 / 4, 0, 0, 0], [-33 / 50, 121 / 100, 0, 0],   # sdirk3.py:10-12
                  [239 / 400, -71 / 100, 5 / 16, 0], [-1 / 48, -17 / 66, 235 / 528, -1 / 6]])
C3 = np.array([0., 1 / 4, 4 / 5, 1., 1.])  # sdirk3.py:13


def _sav_stage(m: OracleModel, rhs, scalar_rhs, conv, lifting, dt, predictor, d, viscosity, order, gamma):
    """One mr-SAV stage as shared by ``sdirk2_mrsav.py:21-59`` and
    ``sdirk3_mrsav.py:29-57``: two Stokes columns, alpha/beta with the
    negative-energy guard, Phi, recombination, scalar residual, full momentum
    defect and the 1e-8 gates."""
    solved = m.solve_columns([rhs, conv], mass=1.0, viscosity=viscosity)
    V, W = solved[0].velocity, solved[1].velocity
    alpha = m.pair(conv, V) + lifting
    beta = m.pair(conv, W)
    if beta < 0.0:
        if beta < -1e-12 * (1 + m.cauchy_scale(conv, W)):
            raise RuntimeError("Negative Stokes response energy")
    beta = max(beta, 0.0)
    upd = solve_scalar_stage(predictor, dt, d, scalar_rhs, alpha, beta, order=order)
    r, coupling = upd.r, upd.coupling
    velocity = m.combine((1.0, V), (-dt * coupling, W))
    pressure = m.combine((1.0 / dt, solved[0].pressure), (-coupling, solved[1].pressure))
    scalar = d * r - scalar_rhs + dt * upd.factor * (m.pair(conv, velocity) + lifting)
    scalar_residual = abs(scalar) / (1 + abs(scalar_rhs) + abs(r))
    kv = m.apply_K(velocity)
    defect = m.combine((1.0, velocity), (viscosity, kv), (dt, m.apply_G(pressure)), (-1.0, rhs),
                       (dt * coupling, conv))
    residual = m.residual(defect, rhs, conv, dt * abs(coupling))
    phys, cont = m.stage_divergences(velocity)
    if (not np.isfinite([residual, scalar_residual, cont]).all() or residual > 1e-8
            or scalar_residual > 1e-8 or cont > 1e-8 * (1 + m.max_abs(velocity))):
        raise RuntimeError(f"SAV stage residuals {residual}, {scalar_residual}, divergence {cont}")
    st = upd.record(m.stage(pressure, residual, phys, r, scalar_residual=scalar_residual,
                            continuity_residual=cont))
    return velocity, st, kv


class SDIRK2MRSAV:
    """``solver/schemes/sdirk2_mrsav.py:15-75``."""
    name = "sdirk2_mrsav"

    def __init__(self, gamma: float = 1.0):
        if not np.isfinite(gamma) or gamma < 0:
            raise ValueError("gamma must be finite and nonnegative")
        self.gamma = gamma

    def step(self, m: OracleModel, s: State, dt: float) -> Trial:
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError("Invalid step size")
        g, visc = self.gamma, m.nu * ETA * dt
        d = 1 + g * ETA * dt
        old = m.vector(s)
        n0, l0 = m.nonlinear_with_lifting(old)
        f0 = m.force(s.t)
        first, s1, k1 = _sav_stage(m, m.combine((1.0, old), (ETA * dt, f0)), s.r, m.combine((ETA, n0)),
                                   ETA * l0, dt, s.r, d, visc, 2, g)
        n1, l1 = m.nonlinear_with_lifting(first)
        f1 = m.force(s.t + ETA * dt)
        rhs = m.combine((1.0, first), (-m.nu * dt * (1 - 2 * ETA), k1), (-dt, f0), (dt * (1 - DELTA), f1))
        second, s2, _ = _sav_stage(m, rhs, (1 - g * dt * (1 - 2 * ETA)) * s1.r,
                                   m.combine((-1.0, n0), (1 - DELTA, n1)), -l0 + (1 - DELTA) * l1,
                                   dt, s1.r, d, visc, 2, g)
        emb = m.combine((1.0 - 1.0 / ETA, old), (1.0 / ETA, first))
        return Trial(m.state(s.t + dt, second, s2.r), [s1, s2], emb)


def _known_terms(m, nonlin, forces, i):  # sdirk3.py:22-28
    conv = m.combine(*[(DHAT3[i, j], nonlin[j][0]) for j in range(i + 1)])
    lifting = float(sum(DHAT3[i, j] * nonlin[j][1] for j in range(i + 1)))
    force = m.combine(*[(DHAT3[i, j], forces[j]) for j in range(i + 1)])
    return conv, force, lifting


def _embedded3(m, vs):  # sdirk3.py:16-19
    return m.combine((2 / 3, vs[0]), (-128 / 99, vs[1]), (50 / 33, vs[2]), (1 / 9, vs[3]))


class SDIRK3MRSAV:
    """``solver/schemes/sdirk3_mrsav.py:11-65``."""
    name = "sdirk3_mrsav"

    def __init__(self, gamma: float = 1.0):
        if not np.isfinite(gamma) or gamma < 0:
            raise ValueError("gamma must be finite and nonnegative")
        self.gamma = gamma

    def step(self, m: OracleModel, s: State, dt: float) -> Trial:
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError("Invalid step size")
        vs = [m.vector(s)]
        lin, scal, stages = [], [s.r], []
        nonlin = [m.nonlinear_with_lifting(vs[0])]
        forces = [m.force(s.t + C3[j] * dt) for j in range(4)]
        for i in range(4):
            conv, force, lifting = _known_terms(m, nonlin, forces, i)
            rhs = m.combine((1.0, vs[-1]), (dt, force), *[(-m.nu * dt * D3[i, j], lin[j]) for j in range(i)])
            srhs = scal[-1] - self.gamma * dt * sum(D3[i, j] * scal[j + 1] for j in range(i))
            vel, st, kv = _sav_stage(m, rhs, srhs, conv, lifting, dt, scal[-1], 1 + self.gamma * dt * D3[i, i],
                                     m.nu * dt * D3[i, i], 3, self.gamma)
            vs.append(vel)
            lin.append(kv)
            if i < 3:
                nonlin.append(m.nonlinear_with_lifting(vel))
            scal.append(st.r)
            stages.append(st)
        return Trial(m.state(s.t + dt, vs[-1], scal[-1]), stages, _embedded3(m, vs))


class SDIRK2:
    """Plain incremental IMEX-SDIRK2 (``solver/schemes/sdirk2.py:17-43``)."""
    name = "sdirk2"

    def step(self, m, s, dt):
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError("Invalid step size")
        old = m.vector(s)
        n0 = m.nonlinear(old)
        f0 = m.force(s.t)
        visc = m.nu * ETA * dt
        first = m.solve(m.combine((1.0, old), (ETA * dt, f0), (-ETA * dt, n0)), mass=1.0, viscosity=visc)
        f1 = m.force(s.t + ETA * dt)
        n1 = m.nonlinear(first.velocity)
        rhs = m.combine((1.0, first.velocity), (-m.nu * dt * (1 - 2 * ETA), m.apply_K(first.velocity)),
                        (-dt, f0), (dt * (1 - DELTA), f1), (dt, n0), (-dt * (1 - DELTA), n1))
        second = m.solve(rhs, mass=1.0, viscosity=visc)
        stages = []
        for sol in (first, second):
            phys, cont = m.stage_divergences(sol.velocity)
            stages.append(m.stage(m.combine((1.0 / dt, sol.pressure)), sol.residual, phys,
                                  continuity_residual=cont))
        emb = m.combine((1.0 - 1.0 / ETA, old), (1.0 / ETA, first.velocity))
        return Trial(m.state(s.t + dt, second.velocity), stages, emb)


class SDIRK3:
    """Plain four-stage IMEX-SDIRK3 (``solver/schemes/sdirk3.py:31-57``)."""
    name = "sdirk3"

    def step(self, m, s, dt):
        if not np.isfinite(dt) or dt <= 0:
            raise ValueError("Invalid step size")
        vs = [m.vector(s)]
        lin, stages = [], []
        nonlin = [m.nonlinear_with_lifting(vs[0])]
        forces = [m.force(s.t + C3[j] * dt) for j in range(4)]
        for i in range(4):
            conv, force, _ = _known_terms(m, nonlin, forces, i)
            rhs = m.combine((1.0, vs[-1]), (dt, force), (-dt, conv),
                            *[(-m.nu * dt * D3[i, j], lin[j]) for j in range(i)])
            sol = m.solve(rhs, mass=1.0, viscosity=m.nu * dt * D3[i, i])
            vs.append(sol.velocity)
            if i < 3:
                lin.append(m.apply_K(sol.velocity))
                nonlin.append(m.nonlinear_with_lifting(sol.velocity))
            phys, cont = m.stage_divergences(sol.velocity)
            stages.append(m.stage(m.combine((1 / dt, sol.pressure)), sol.residual, phys,
                                  continuity_residual=cont))
        return Trial(m.state(s.t + dt, vs[-1]), stages, _embedded3(m, vs))


class IMEXEuler:
    """``solver/schemes/imex_euler.py:10-32``."""
    name = "imex_euler"

    def step(self, m, s, dt):
        if not np.isfinite(dt) or dt <= 0 or not np.isfinite(s.t):
            raise ValueError("Invalid step size or state time")
        old = m.vector(s)
        conv = m.nonlinear(old)
        rhs = m.combine((1.0, old), (dt, m.force(s.t)), (-dt, conv))
        sol = m.solve(rhs, mass=1.0, viscosity=m.nu * dt)
        vel = sol.velocity
        pres = m.combine((1 / dt, sol.pressure))
        defect = m.combine((1.0, vel), (m.nu * dt, m.apply_K(vel)), (dt, m.apply_G(pres)), (-1.0, rhs))
        res = m.residual(defect, rhs)
        phys, cont = m.stage_divergences(vel)
        if (not np.isfinite([res, phys, cont, m.max_abs(vel), m.max_abs(pres)]).all()
                or res > 1e-8 or cont > 1e-8 * (1 + m.max_abs(vel))):
            raise RuntimeError(f"IMEX Euler residual {res}, divergence {cont}")
        return Trial(m.state(s.t + dt, vel), [m.stage(pres, res, phys, continuity_residual=cont)])


class IMEXEulerMRSAV:
    """``solver/schemes/imex_euler_mrsav.py:11-53``."""
    name = "imex_euler_mrsav"

    def __init__(self, gamma: float = 1.0):
        if not np.isfinite(gamma) or gamma < 0:
            raise ValueError("gamma must be finite and nonnegative")
        self.gamma = gamma

    def step(self, m, s, dt):
        if not np.isfinite(dt) or dt <= 0 or not np.isfinite([s.t, s.r]).all():
            raise ValueError("Invalid step size or scalar state")
        old = m.vector(s)
        conv, lifting = m.nonlinear_with_lifting(old)
        rhs = m.combine((1.0, old), (dt, m.force(s.t)))
        solved = m.solve_columns([rhs, conv], mass=1.0, viscosity=m.nu * dt)
        V, W = solved[0].velocity, solved[1].velocity
        alpha = m.pair(conv, V) + lifting
        beta = m.pair(conv, W)
        if beta < 0.0 and beta < -1e-12 * (1 + m.cauchy_scale(conv, W)):
            raise RuntimeError("Negative Stokes response energy")
        beta = max(beta, 0.0)
        smass = 1 + self.gamma * dt
        upd = solve_scalar_stage(s.r, dt, smass, s.r, alpha, beta, order=1)
        r, corr = upd.r, upd.coupling
        vel = m.combine((1.0, V), (-dt * corr, W))
        pres = m.combine((1 / dt, solved[0].pressure), (-corr, solved[1].pressure))
        scalar = smass * r - s.r + dt * (m.pair(conv, vel) + lifting)
        sres = abs(scalar) / (1 + abs(s.r) + abs(r))
        defect = m.combine((1.0, vel), (m.nu * dt, m.apply_K(vel)), (dt, m.apply_G(pres)), (-1.0, rhs),
                           (dt * corr, conv))
        res = m.residual(defect, rhs, conv, dt * abs(corr))
        phys, cont = m.stage_divergences(vel)
        if (not np.isfinite([r, res, sres, phys, cont, m.max_abs(vel), m.max_abs(pres)]).all()
                or res > 1e-8 or sres > 1e-8 or cont > 1e-8 * (1 + m.max_abs(vel))):
            raise RuntimeError(f"IMEX Euler SAV residuals {res}, {sres}, divergence {cont}")
        st = upd.record(m.stage(pres, res, phys, r, scalar_residual=sres, continuity_residual=cont))
        return Trial(m.state(s.t + dt, vel, r), [st])


_SCHEMES = {"sdirk2": lambda g: SDIRK2(), "sdirk2_mrsav": SDIRK2MRSAV, "sdirk3": lambda g: SDIRK3(),
            "sdirk3_mrsav": SDIRK3MRSAV, "imex_euler": lambda g: IMEXEuler(),
            "imex_euler_mrsav": IMEXEulerMRSAV}


def make_scheme(name: str, gamma: float = 1.0):  # solver/schemes/registry.py:44-53
    if name not in _SCHEMES:
        raise ValueError(f"Unknown scheme: {name}")
    return _SCHEMES[name](gamma)


# --------------------------------------------------------------------- driver
def schedule_nodes(t0: float, seq: np.ndarray) -> np.ndarray:
    """Compensated node times (``solver/schedule.py:7-19``)."""
    nodes = np.empty(seq.size + 1)
    nodes[0] = t0
    total, corr = float(t0), 0.0
    for k, h in enumerate(seq, start=1):
        inc = float(h) - corr
        new = total + inc
        corr = (new - total) - inc
        total = new
        nodes[k] = total
    return nodes


def nearest_node_indices(nodes, requests):  # solver/schedule.py:22-29
    out = []
    for t in requests:
        dist = np.abs(nodes - t)
        tie = 8 * np.finfo(float).eps * max(abs(t), float(np.max(np.abs(nodes))), np.finfo(float).tiny)
        out.append(int(np.flatnonzero(dist <= dist.min() + tie)[0]))
    return out


@dataclass
class Result:  # solver/integrate.py:12-25
    final: State
    times: list
    diagnostics: list
    stages: list = field(default_factory=list)
    final_stages: list = field(default_factory=list)
    status: str = "complete"
    error: str = ""
    seconds: float = 0.0


def integrate(m, scheme, initial: State, steps) -> Result:
    """Fixed/prescribed-step loop (``solver/integrate.py:47-100``), without
    snapshots and observers: finiteness checks, diagnostics, failure prefix."""
    seq = np.asarray(steps, dtype=float)
    if seq.ndim != 1 or seq.size == 0 or np.any(seq <= 0) or not np.isfinite(seq).all():
        raise ValueError("Invalid step sequence")
    state = initial
    res = Result(initial, [initial.t], [m.diagnostics(initial)])
    start = perf_counter()
    for dt in seq:
        try:
            trial = scheme.step(m, state, float(dt))
            if not np.isfinite(m.vector(trial.state)).all() or not np.isfinite(trial.state.r):
                raise FloatingPointError("Nonfinite trial state")
            diag = m.diagnostics(trial.state)
            if not all(np.isfinite(v) for v in diag.values()):
                raise FloatingPointError("Nonfinite diagnostic")
            state = trial.state
            res.final = state
            res.times.append(state.t)
            res.diagnostics.append(diag)
            res.final_stages = trial.stages
            res.stages.append([stage_diagnostics(s) for s in trial.stages])
        except Exception as err:  # integrate.py:90-93
            res.status = "failed"
            res.error = f"{type(err).__name__}: {err}"
            break
    res.seconds = perf_counter() - start
    return res
