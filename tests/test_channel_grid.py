"""ChannelGrid host layout (no GPU): grid.py semantics and errors
(tests/core/test_channel_operators.py:7-25)."""
import numpy as np
import pytest

from helpers import load_package


@pytest.fixture(scope="module")
def ch():
    from importlib import import_module
    return import_module(load_package().__name__ + ".channel")


def test_layout_roundtrip_periodic_weights_and_loads(ch):
    grid = ch.ChannelGrid(7, 5, 2., .7)
    w = np.random.default_rng(13).normal(size=grid.size)
    u, v = grid.unpack(w)
    np.testing.assert_array_equal(u[:, 0], u[:, -1])
    np.testing.assert_array_equal(v[[0, -1]], 0.)
    np.testing.assert_array_equal(grid.pack(u, v), w)
    assert grid.inner(w, w) == pytest.approx(grid.area * (np.sum(u[:, :-1] ** 2) + np.sum(v[1:-1] ** 2)))
    v[[0, -1]] = 2.
    np.testing.assert_array_equal(grid.pack_load(u, v), w)
    with pytest.raises(ValueError, match="wall"):
        grid.pack(u, v)
    u[:, -1] += 1.
    with pytest.raises(ValueError, match="periodic"):
        grid.pack_load(u, v)
    with pytest.raises(ValueError):
        grid.unpack(w.astype(complex))
    u[0, 0] = np.nan
    with pytest.raises(ValueError, match="finite"):
        grid.pack_load(u, v)


@pytest.mark.parametrize("args", [(True, 5), (2, 5), (5, 4, 0.), (5, 4, 1., np.inf)])
def test_invalid_grids(ch, args):
    with pytest.raises(ValueError):
        ch.ChannelGrid(*args)


def test_curl_is_discretely_divergence_free(ch):
    grid = ch.ChannelGrid(7, 5, 1.3, .8)
    x, y = grid.coordinates("vertex")
    psi = np.sin(2 * np.pi * x / grid.lx) * np.sin(np.pi * y / grid.ly) ** 2
    psi[[0, -1]] = 0.
    u, v = grid.unpack(grid.curl(psi))
    div = np.diff(u, axis=1) / grid.hx + np.diff(v, axis=0) / grid.hy
    assert np.abs(div).max() < 1e-13
    assert grid.metadata()["boundary"] == "periodic_x_no_slip_y"
