"""The channel-MAC oracle against fixtures generated by the reference itself
(tests/golden/make_golden.py, ``channel``)."""
import numpy as np
import pytest

from helpers import golden
from oracle import channel_oracle as CO


@pytest.fixture(scope="module")
def d():
    return golden("channel")


@pytest.mark.parametrize("shape", [(7, 5), (8, 6), (17, 9)])
@pytest.mark.parametrize("k", [0, 1, 2])
def test_fft_solve_matches_reference(d, shape, k):
    nx, ny = shape
    tag = f"solve_{nx}x{ny}_{k}"
    g = CO.ChannelGridOracle(nx, ny, 2.3, .8)
    mass, alpha = d[f"{tag}_shift"]
    vel, pres = CO.fft_solve(g, d[f"{tag}_loads"], float(mass), float(alpha))
    np.testing.assert_allclose(vel, d[f"{tag}_vel"], rtol=1e-10, atol=1e-11)
    np.testing.assert_allclose(pres, d[f"{tag}_pres"], rtol=1e-10, atol=1e-11)


def test_operators_and_convection_match_reference(d):
    g = CO.ChannelGridOracle(9, 7, 2., .8)
    K, D, G = CO.operators(g)
    w = d["conv_w"]
    np.testing.assert_allclose(K @ w, d["conv_K"], rtol=1e-13, atol=1e-12)
    np.testing.assert_allclose(D @ w, d["conv_D"], rtol=1e-13, atol=1e-12)
    np.testing.assert_allclose(G @ d["conv_p"], d["conv_G"], rtol=1e-13, atol=1e-12)
    u, v = g.unpack(w)
    np.testing.assert_allclose(g.pack(*CO.convection(u, v, g.hx, g.hy)), d["conv_n"], rtol=1e-13, atol=1e-12)
