"""NumPy/SciPy restatement of the reference's channel MAC path (test oracle).

Periodic x, stationary no-slip y (``solver/channel/*.py`` of the
HaifengWang1031/MAC-mr-SAV-RK project).  Restated here: the packed layout
(grid.py:64-77), the sparse operators (operators.py:9-25), the skew periodic
convection (kernels.py:9-41, vectorised), and the FFT Stokes solve
(fft_stokes.py:94-137: orthonormal rFFT along x, one saddle solve per x
mode, zero mode by a tridiagonal solve and a pressure cumulative sum).  The
per-mode systems are solved densely here (small test grids only).

Nothing here runs on a GPU; it is the CPU checker only.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
from scipy.fft import irfft, rfft


@dataclass(frozen=True)
class ChannelGridOracle:
    nx: int
    ny: int
    lx: float = 1.0
    ly: float = 1.0

    @property
    def hx(self):
        return self.lx / self.nx

    @property
    def hy(self):
        return self.ly / self.ny

    @property
    def nu(self):
        return self.nx * self.ny

    @property
    def size(self):
        return self.nx * self.ny + self.nx * (self.ny - 1)

    @property
    def np(self):
        return self.nx * self.ny

    def pack(self, u, v):  # grid.py:57-68
        return np.concatenate((u[:, :self.nx].ravel(), v[1:-1, :].ravel()))

    def unpack(self, w):  # grid.py:70-77
        u = np.empty((self.ny, self.nx + 1))
        u[:, :self.nx] = w[:self.nu].reshape(self.ny, self.nx)
        u[:, -1] = u[:, 0]
        v = np.zeros((self.ny + 1, self.nx))
        v[1:-1, :] = w[self.nu:].reshape(self.ny - 1, self.nx)
        return u, v


def _lap(n: int, h: float, wall: bool):  # solver/mac/operators.py:6-9
    d = np.full(n, 2.0)
    if wall:
        d[[0, -1]] = 3.0
    return sp.diags([-np.ones(n - 1), d, -np.ones(n - 1)], [-1, 0, 1], format="csr") / h ** 2


def operators(g: ChannelGridOracle):
    """(K, D, G) of operators.py:9-25."""
    nx, ny = g.nx, g.ny
    rows = np.arange(nx)
    fwd = sp.csr_matrix((np.ones(nx), (rows, (rows + 1) % nx)), shape=(nx, nx))
    dx = (fwd - sp.eye(nx, format="csr")) / g.hx
    kx = dx.T @ dx
    ku = sp.kron(sp.eye(ny), kx) + sp.kron(_lap(ny, g.hy, True), sp.eye(nx))
    kv = sp.kron(sp.eye(ny - 1), kx) + sp.kron(_lap(ny - 1, g.hy, False), sp.eye(nx))
    K = sp.block_diag([ku, kv], format="csr")
    dy = sp.diags([np.ones(ny - 1), -np.ones(ny - 1)], [0, -1], shape=(ny, ny - 1), format="csr") / g.hy
    D = sp.hstack([sp.kron(sp.eye(ny), dx), sp.kron(dy, sp.eye(nx))], format="csr")
    return K, D, -D.T.tocsr()


def convection(u, v, hx, hy):
    """Skew dual-cell fluxes, periodic x and odd tangential y extension (kernels.py:9-41)."""
    q = u[:, :-1]
    qe, qw = np.roll(q, -1, 1), np.roll(q, 1, 1)
    east, west = .5 * (q + qe), .5 * (q + qw)
    north = .5 * (v[1:] + np.roll(v[1:], 1, 1))
    south = .5 * (v[:-1] + np.roll(v[:-1], 1, 1))
    un = np.vstack([q[1:], -q[-1:]])
    us = np.vstack([-q[:1], q[:-1]])
    cu = (east * east - west * west) / hx + (north * .5 * (q + un) - south * .5 * (q + us)) / hy
    cu -= .5 * q * ((east - west) / hx + (north - south) / hy)
    qv = v[1:-1]
    west_v = .5 * (q[:-1] + q[1:])
    east_v = np.roll(west_v, -1, 1)
    north_v, south_v = .5 * (qv + v[2:]), .5 * (qv + v[:-2])
    cv = (east_v * .5 * (qv + np.roll(qv, -1, 1)) - west_v * .5 * (qv + np.roll(qv, 1, 1))) / hx
    cv += (north_v * north_v - south_v * south_v) / hy
    cv -= .5 * qv * ((east_v - west_v) / hx + (north_v - south_v) / hy)
    cu_full = np.column_stack([cu, cu[:, 0]])
    cv_full = np.vstack([np.zeros_like(v[:1]), cv, np.zeros_like(v[:1])])
    return cu_full, cv_full


def fft_solve(g: ChannelGridOracle, rhs: np.ndarray, mass: float, visc: float):
    """FFTStokes.solve (fft_stokes.py:94-137) with dense per-mode solves.
    rhs (size,) or (size, c); returns (velocity, pressure (ny, nx[, c]))."""
    force = rhs if rhs.ndim == 2 else rhs[:, None]
    c = force.shape[1]
    nx, ny = g.nx, g.ny
    fu = rfft(force[:g.nu].reshape(ny, nx, c), axis=1, norm="ortho")
    fv = rfft(force[g.nu:].reshape(ny - 1, nx, c), axis=1, norm="ortho")
    nm = nx // 2 + 1
    uh = np.zeros((ny, nm, c), complex)
    vh = np.zeros((ny - 1, nm, c), complex)
    ph = np.zeros((ny, nm, c), complex)
    ku, kv = _lap(ny, g.hy, True).toarray(), _lap(ny - 1, g.hy, False).toarray()
    dy = (np.eye(ny, ny - 1) - np.eye(ny, ny - 1, -1)) / g.hy
    uh[:, 0] = np.linalg.solve(mass * np.eye(ny) + visc * ku, fu[:, 0])
    ph[1:, 0] = g.hy * np.cumsum(fv[:, 0], axis=0)
    ph[:, 0] -= ph[:, 0].mean(axis=0)
    for m in range(1, nm):
        theta = 2 * np.pi * m / nx
        d = complex(-2 / g.hx) if (nx % 2 == 0 and m == nx // 2) else (np.exp(1j * theta) - 1) / g.hx
        lam = 4 * np.sin(theta / 2) ** 2 / g.hx ** 2
        hu = (mass + visc * lam) * np.eye(ny) + visc * ku
        hv = (mass + visc * lam) * np.eye(ny - 1) + visc * kv
        a = np.block([[hu, np.zeros((ny, ny - 1)), -np.conj(d) * np.eye(ny)],
                      [np.zeros((ny - 1, ny)), hv, -dy.T],
                      [-d * np.eye(ny), -dy, np.zeros((ny, ny))]])
        b = np.vstack([fu[:, m], fv[:, m], np.zeros((ny, c))])
        x = np.linalg.solve(a, b)
        uh[:, m], vh[:, m], ph[:, m] = x[:ny], x[ny:2 * ny - 1], x[2 * ny - 1:]
    vel = np.concatenate([irfft(uh, n=nx, axis=1, norm="ortho").reshape(-1, c),
                          irfft(vh, n=nx, axis=1, norm="ortho").reshape(-1, c)])
    pres = irfft(ph, n=nx, axis=1, norm="ortho")
    pres -= pres.mean(axis=(0, 1), keepdims=True)
    if rhs.ndim == 1:
        return vel[:, 0], pres[:, :, 0]
    return vel, pres
