"""Uniform MAC layout (the reference's ``MACGrid``, solver/mac/grid.py:9-71).

Host-side bookkeeping only: shapes, spacings, pack/unpack between the full
face arrays and the packed free vector, and the area-weighted inner product.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class MACGrid:
    nx: int
    ny: int
    lx: float = 1.0
    ly: float = 1.0

    def __post_init__(self) -> None:  # grid.py:15-19
        if isinstance(self.nx, bool) or isinstance(self.ny, bool) or not isinstance(self.nx, int) \
                or not isinstance(self.ny, int):
            raise ValueError("nx, ny must be integers")
        if min(self.nx, self.ny) < 3 or not np.isfinite([self.lx, self.ly]).all() or min(self.lx, self.ly) <= 0:
            raise ValueError("Require nx,ny >= 3 and positive finite domain lengths")

    @property
    def hx(self) -> float:
        return self.lx / self.nx

    @property
    def hy(self) -> float:
        return self.ly / self.ny

    @property
    def nu(self) -> int:
        return (self.nx - 1) * self.ny

    @property
    def nv(self) -> int:
        return self.nx * (self.ny - 1)

    @property
    def size(self) -> int:
        return self.nu + self.nv

    @property
    def np(self) -> int:
        return self.nx * self.ny

    @property
    def area(self) -> float:
        return self.hx * self.hy

    def coordinates(self, field: str) -> tuple[np.ndarray, np.ndarray]:
        """Meshgrids of face / cell / vertex positions (grid.py:36-50)."""
        hx, hy, nx, ny = self.hx, self.hy, self.nx, self.ny
        if field == "u":
            x, y = np.arange(nx + 1, dtype=float) * hx, (np.arange(ny, dtype=float) + .5) * hy
        elif field == "v":
            x, y = (np.arange(nx, dtype=float) + .5) * hx, np.arange(ny + 1, dtype=float) * hy
        elif field == "p":
            x, y = (np.arange(nx, dtype=float) + .5) * hx, (np.arange(ny, dtype=float) + .5) * hy
        elif field == "vertex":
            x, y = np.arange(nx + 1, dtype=float) * hx, np.arange(ny + 1, dtype=float) * hy
        else:
            raise ValueError(f"Unknown field {field}")
        return np.meshgrid(x, y)

    def pack(self, u: np.ndarray, v: np.ndarray) -> np.ndarray:
        if u.shape != (self.ny, self.nx + 1) or v.shape != (self.ny + 1, self.nx):
            raise ValueError("Incorrect MAC array shapes")
        if np.any(u[:, [0, -1]] != 0) or np.any(v[[0, -1], :] != 0):
            raise ValueError("Normal boundary velocities must be zero")
        return np.concatenate((u[:, 1:-1].ravel(), v[1:-1, :].ravel()))

    def unpack(self, velocity: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        if velocity.shape != (self.size,):
            raise ValueError("Incorrect free-vector shape")
        u = np.zeros((self.ny, self.nx + 1))
        v = np.zeros((self.ny + 1, self.nx))
        u[:, 1:-1] = velocity[:self.nu].reshape(self.ny, self.nx - 1)
        v[1:-1, :] = velocity[self.nu:].reshape(self.ny - 1, self.nx)
        return u, v

    def inner(self, a: np.ndarray, b: np.ndarray) -> float:
        return float(self.area * np.dot(a, b))

    def norm(self, a: np.ndarray) -> float:
        return float(np.sqrt(self.inner(a, a)))


def grid_of(obj) -> MACGrid:
    """Accepts a grid, or an operators object carrying ``.grid`` (the reference's
    ``MACOperators``), and returns this package's MACGrid."""
    g = getattr(obj, "grid", obj)
    return g if isinstance(g, MACGrid) else MACGrid(int(g.nx), int(g.ny), float(g.lx), float(g.ly))
