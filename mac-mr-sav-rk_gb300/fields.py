"""Seeded synthetic initial fields for the no-slip MAC cavity workloads.

The initial velocity is the discrete curl of a stream function sampled at cell
corners, so its discrete divergence is exactly zero (the construction of the
reference's ``tests/references/mac.py:14-21``, with a random modal sum):

    psi = sin^2(pi x/lx) sin^2(pi y/ly) * sum_{k,l<=K} a_kl sin(k pi x/lx) sin(l pi y/ly)

with ``a_kl ~ N(0, (k^2+l^2)^-2)`` (standard deviation ``1/(k^2+l^2)``) drawn
from ``numpy.random.default_rng(seed)`` in (k, l) row-major order.  Then
``u = diff(psi, axis=0)/hy`` and ``v = -diff(psi, axis=1)/hx`` with psi zeroed
on the boundary, and the normal wall faces are zero by construction.
"""
from __future__ import annotations

import numpy as np


def stream_function(nx: int, ny: int, lx: float, ly: float, modes: int, seed: int) -> np.ndarray:
    """psi at the (ny+1, nx+1) cell corners."""
    rng = np.random.default_rng(seed)
    k = np.arange(1, modes + 1, dtype=float)
    amp = np.empty((modes, modes))
    for a in range(modes):          # (k, l) row-major draw order
        for b in range(modes):
            amp[a, b] = rng.normal(0.0, 1.0 / (k[a] ** 2 + k[b] ** 2))
    x = np.arange(nx + 1, dtype=float) * (lx / nx)
    y = np.arange(ny + 1, dtype=float) * (ly / ny)
    sx = np.sin(np.pi * np.outer(k, x) / lx)        # (K, nx+1)
    sy = np.sin(np.pi * np.outer(k, y) / ly)        # (K, ny+1)
    series = sy.T @ amp.T @ sx                      # sum_{k,l} a_kl sin(k.x) sin(l.y), (ny+1, nx+1)
    envelope = np.outer(np.sin(np.pi * y / ly) ** 2, np.sin(np.pi * x / lx) ** 2)
    psi = envelope * series
    psi[[0, -1], :] = 0.0
    psi[:, [0, -1]] = 0.0
    return psi


def curl_velocity(nx: int, ny: int, lx: float, ly: float, modes: int, seed: int) -> tuple[np.ndarray, np.ndarray]:
    """Full MAC face arrays u (ny, nx+1) and v (ny+1, nx), exactly divergence free."""
    psi = stream_function(nx, ny, lx, ly, modes, seed)
    u = np.diff(psi, axis=0) / (ly / ny)
    v = -np.diff(psi, axis=1) / (lx / nx)
    return u, v


def packed_curl_velocity(nx: int, ny: int, lx: float, ly: float, modes: int, seed: int) -> np.ndarray:
    """The packed free vector [u[:,1:-1].ravel(), v[1:-1,:].ravel()]."""
    u, v = curl_velocity(nx, ny, lx, ly, modes, seed)
    return np.concatenate((u[:, 1:-1].ravel(), v[1:-1, :].ravel()))
