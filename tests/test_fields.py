"""The seeded synthetic initial fields (host code, no GPU): the discrete curl
of the corner stream function is divergence free under the reference's D
(the oracle's restatement), zero on the normal wall faces, and a pure
function of its seed."""
import numpy as np
import pytest

import oracle as O
from helpers import load_package


@pytest.fixture(scope="module")
def fields():
    from importlib import import_module
    return import_module(load_package().__name__ + ".fields")


@pytest.mark.parametrize("shape", [(9, 7, 1.3, 0.8), (64, 64, 1.0, 1.0), (96, 64, 1.5, 1.0), (32, 128, 0.25, 1.0)],
                         ids=lambda s: f"{s[0]}x{s[1]}")
def test_curl_field_is_divergence_free_with_zero_normal_walls(fields, shape):
    nx, ny, lx, ly = shape
    u, v = fields.curl_velocity(nx, ny, lx, ly, 8, 5)
    assert u.shape == (ny, nx + 1) and v.shape == (ny + 1, nx)
    np.testing.assert_array_equal(u[:, [0, -1]], 0.0)
    np.testing.assert_array_equal(v[[0, -1], :], 0.0)
    g = O.Grid(nx, ny, lx, ly)
    x = fields.packed_curl_velocity(nx, ny, lx, ly, 8, 5)
    assert x.shape == (g.size,)
    np.testing.assert_array_equal(x, g.pack(u, v))
    scale = np.abs(x).max() / min(g.hx, g.hy)
    assert np.abs(O.apply_D(g, x)).max() <= 1e-13 * scale


def test_curl_field_is_a_function_of_its_seed(fields):
    a = fields.packed_curl_velocity(48, 32, 1.5, 1.0, 6, 7)
    np.testing.assert_array_equal(a, fields.packed_curl_velocity(48, 32, 1.5, 1.0, 6, 7))
    b = fields.packed_curl_velocity(48, 32, 1.5, 1.0, 6, 8)
    assert np.linalg.norm(a - b) > 0.1 * np.linalg.norm(a)
    # the stream function at the cell corners, zero on the boundary
    psi = fields.stream_function(48, 32, 1.5, 1.0, 6, 7)
    assert psi.shape == (33, 49) and np.all(psi[[0, -1], :] == 0) and np.all(psi[:, [0, -1]] == 0)
