"""GPU channel MAC (periodic x, no-slip y): the FFT Stokes backend, operators,
convection and the model seam against the reference's fixtures and the
behaviours its own tests pin (tests/core/test_channel_*.py)."""
import numpy as np
import pytest

import oracle as O
from helpers import golden, load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ch():
    from importlib import import_module
    return import_module(load_package().__name__ + ".channel")


@pytest.fixture(scope="module")
def d():
    return golden("channel")


@pytest.mark.parametrize("shape", [(7, 5), (8, 6), (17, 9)])
@pytest.mark.parametrize("k", [0, 1, 2])
def test_fft_solve_matches_reference(ch, d, shape, k):
    nx, ny = shape
    tag = f"solve_{nx}x{ny}_{k}"
    grid = ch.ChannelGrid(nx, ny, 2.3, .8)
    model = ch.ChannelModel(grid, .1, backend="fft")
    mass, alpha = (float(x) for x in d[f"{tag}_shift"])
    sol = model.backend.solve(d[f"{tag}_loads"], mass=mass, viscosity=alpha)
    np.testing.assert_allclose(sol.velocity, d[f"{tag}_vel"], rtol=2e-12, atol=2e-12)
    np.testing.assert_allclose(sol.pressure, d[f"{tag}_pres"], rtol=2e-12, atol=2e-12)
    loads = d[f"{tag}_loads"]
    defect = mass * sol.velocity + alpha * (model.ops.K @ sol.velocity) \
        + model.ops.G @ sol.pressure.reshape(grid.np, 2) - loads
    assert np.abs(defect).max() < 2e-12
    assert sol.divergence_inf < 1e-11 and sol.residual < 1e-11


def test_operators_convection_and_skew_pairing(ch, d):
    grid = ch.ChannelGrid(9, 7, 2., .8)
    model = ch.ChannelModel(grid, .1)
    w = d["conv_w"]
    np.testing.assert_allclose(model.apply_K(w).cpu().numpy(), d["conv_K"], rtol=1e-13, atol=1e-11)
    np.testing.assert_allclose(model.apply_D(w).cpu().numpy(), d["conv_D"], rtol=1e-13, atol=1e-12)
    np.testing.assert_allclose(model.apply_G(d["conv_p"]).cpu().numpy(), d["conv_G"], rtol=1e-13, atol=1e-12)
    n = model.nonlinear(w)
    np.testing.assert_allclose(n.cpu().numpy(), d["conv_n"], rtol=1e-13, atol=1e-12)
    assert abs(model.inner(n, w)) < 2e-13 * max(1., grid.norm(n.cpu().numpy()) * grid.norm(w))
    p = np.random.default_rng(31).normal(size=grid.np)
    assert np.dot(w, model.ops.G @ p) == pytest.approx(-np.dot(model.ops.D @ w, p), abs=1e-12)
    np.testing.assert_array_equal(model.ops.G @ np.ones(grid.np), 0.)


@pytest.mark.parametrize("nx,ny", [(7, 5), (8, 6)])
def test_laplacian_analytic_modes_including_wall_rows(ch, nx, ny):
    grid = ch.ChannelGrid(nx, ny, 2.3, .8)
    model = ch.ChannelModel(grid, .1)
    xu, yu = grid.coordinates("u")
    xv, yv = grid.coordinates("v")
    u = np.cos(4 * np.pi * xu / grid.lx) * np.sin(np.pi * yu / grid.ly)
    u[:, -1] = u[:, 0]
    v = np.cos(4 * np.pi * xv / grid.lx) * np.sin(np.pi * yv / grid.ly)
    v[[0, -1]] = 0.
    w = grid.pack(u, v)
    eig = 4 * np.sin(2 * np.pi / nx) ** 2 / grid.hx ** 2 + 4 * np.sin(np.pi / (2 * ny)) ** 2 / grid.hy ** 2
    np.testing.assert_allclose(model.ops.K @ w, eig * w, rtol=2e-13, atol=2e-13)


def test_zero_mode_mean_drive_pressure_and_cache(ch):
    """test_channel_fft.py:25-42: gradient loads give zero velocity, the mean
    drive gives the discrete Poiseuille profile, factor cache counters."""
    grid = ch.ChannelGrid(8, 7, 1.2, .9)
    model = ch.ChannelModel(grid, .1, backend="fft", cache_size=2)
    x, y = grid.coordinates("p")
    p = np.cos(2 * np.pi * x / grid.lx) + y - grid.ly / 2
    sol = model.backend.solve(model.apply_G(p).cpu().numpy(), mass=1., viscosity=.1)
    np.testing.assert_allclose(sol.velocity, 0., atol=1e-13)
    np.testing.assert_allclose(sol.pressure, p, atol=1e-13)
    force = grid.pack_load(np.ones((7, 9)), np.zeros((8, 8)))
    sol = model.backend.solve(force, mass=0., viscosity=.1)
    _, yu = grid.coordinates("u")
    expected = (yu * (grid.ly - yu) + grid.hy ** 2 / 4) / .2
    np.testing.assert_allclose(grid.unpack(sol.velocity)[0], expected, atol=1e-12)
    model.backend.solve(force, mass=0., viscosity=.1)
    assert model.backend.factorizations == 2
    model.backend.solve(force, mass=1., viscosity=.2)
    assert len(model.backend.cache) == 2 and model.backend.factorizations == 3


def test_mean_drive_second_order_and_diagnostics(ch):
    """test_channel_model.py:63-80: discrete Poiseuille, second order, and the
    flow-rate / power / dissipation diagnostics."""
    errors = []
    for ny in (8, 16, 32):
        grid = ch.ChannelGrid(5, ny, 2., .7)
        force = grid.pack_load(np.ones((ny, 6)), np.zeros((ny + 1, 5)))
        model = ch.ChannelModel(grid, .13, force=lambda t, f=force: f)
        sol = model.backend.solve(force, mass=0., viscosity=model.nu)
        _, y = grid.coordinates("u")
        exact = y * (grid.ly - y) / (2 * model.nu)
        u, v = grid.unpack(sol.velocity)
        np.testing.assert_allclose(u, exact + grid.hy ** 2 / (8 * model.nu), atol=2e-12)
        np.testing.assert_allclose(v, 0., atol=2e-12)
        errors.append(grid.norm(sol.velocity - grid.pack(exact, v * 0)))
        assert model.max_abs(model.nonlinear(sol.velocity)) < 1e-12
        diag = model.diagnostics(model.state(0., sol.velocity))
        assert diag["flow_rate_spread"] < 1e-12
        assert diag["power"] == pytest.approx(diag["dissipation"], abs=1e-12)
    np.testing.assert_allclose(np.array(errors[:-1]) / errors[1:], 4., rtol=1e-10)


def test_gradient_only_batch_and_wall_normal_load(ch):
    model = ch.ChannelModel(ch.ChannelGrid(7, 5, 1.3, .8), .13, cache_size=2)
    rng = np.random.default_rng(44)
    p = rng.normal(size=(5, 7))
    p -= p.mean()
    b = model.apply_G(p)
    load = rng.normal(size=model.grid.size)
    sols = model.solve_columns([b, load], mass=1., viscosity=.02)
    np.testing.assert_allclose(sols[0].velocity.cpu().numpy(), 0., atol=2e-13)
    np.testing.assert_allclose(sols[0].pressure.cpu().numpy(), p, atol=2e-13)
    assert model.inner(load, sols[1].velocity) >= -1e-13
    grid = ch.ChannelGrid(6, 7, 1.2, .9)
    model = ch.ChannelModel(grid, .1)
    sol = model.backend.solve(grid.pack_load(np.zeros((7, 7)), np.ones((8, 6))), mass=0., viscosity=.1)
    _, y = grid.coordinates("p")
    np.testing.assert_allclose(sol.velocity, 0., atol=1e-13)
    np.testing.assert_allclose(sol.pressure, y - grid.ly / 2, atol=1e-13)


def test_errors_like_reference(ch):
    grid = ch.ChannelGrid(8, 6)
    model = ch.ChannelModel(grid, .1)
    with pytest.raises(ValueError, match="nonnegative"):
        model.backend.solve(np.zeros(grid.size), mass=-1., viscosity=.1)
    with pytest.raises(ValueError, match="Invalid channel FFT RHS"):
        model.backend.solve(np.full(grid.size, np.nan), mass=1., viscosity=.1)
    with pytest.raises(ValueError, match="Invalid channel FFT RHS"):
        model.backend.solve(np.zeros(grid.size + 1), mass=1., viscosity=.1)
    with pytest.raises(ValueError):
        ch.FFTStokes(grid, cache_size=0)
    with pytest.raises(ValueError, match="periodic"):
        u = np.zeros((6, 9))
        u[0, 0] = 1.
        grid.pack_load(u, np.zeros((7, 8)))


@pytest.mark.parametrize("name", ["sdirk2_mrsav", "sdirk3"])
def test_reference_scheme_code_runs_on_gpu_channel(ch, d, name):
    """The oracle's restated schemes (written against the model seam) on the
    GPU ChannelModel reproduce the reference's own FFT-backed run."""
    grid = ch.ChannelGrid(12, 9, 2 * np.pi, 1.)
    model = ch.ChannelModel(grid, .1, backend="fft")
    x0 = d["run_x0"]
    res = O.integrate(model, O.make_scheme(name, 1000.), model.state(0., x0, 1.0 if "mrsav" in name else 0.),
                      [.01, .02, .01])
    assert res.status == "complete", res.error
    np.testing.assert_allclose(model.vector(res.final), d[f"run_{name}_x"], rtol=1e-11, atol=1e-12)
    assert abs(res.final.r - float(d[f"run_{name}_r"])) < 1e-12
    pres = np.array([np.asarray(s.pressure) for s in res.final_stages])
    np.testing.assert_allclose(pres, d[f"run_{name}_p"], rtol=1e-10, atol=1e-11)
    keys = [str(k) for k in d[f"run_{name}_diag_keys"]]
    got = np.array([res.diagnostics[-1][k] for k in keys])
    np.testing.assert_allclose(got, d[f"run_{name}_diag"], rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("nx,ny", [(24, 40), (16, 77)])
def test_spike_solve_multi_step_chunks_match_oracle(ch, nx, ny):
    """Random loads on grids whose banded systems (n = 3 ny - 1 = 119 and 230
    unknowns per mode) span several steps per lane of the warp-partitioned
    substitution, with n not a multiple of 32, and every x mode carrying
    data: velocity and pressure against the oracle's dense per-mode solves."""
    import oracle.channel_oracle as CO
    grid = ch.ChannelGrid(nx, ny, 2.1, .9)
    og = CO.ChannelGridOracle(nx, ny, 2.1, .9)
    model = ch.ChannelModel(grid, .1, backend="fft")
    rng = np.random.default_rng(nx * 1000 + ny)
    loads = rng.normal(size=(grid.size, 2))
    for mass, visc in ((1.0, 2.5e-4), (1.0, .05)):
        sol = model.backend.solve(loads, mass=mass, viscosity=visc)
        vel, pres = CO.fft_solve(og, loads, mass, visc)
        for c in range(2):
            assert np.linalg.norm(sol.velocity[:, c] - vel[:, c]) <= 1e-11 * np.linalg.norm(vel[:, c])
            assert np.linalg.norm(sol.pressure[:, :, c] - pres[:, :, c]) <= 1e-11 * np.linalg.norm(pres[:, :, c])
        assert sol.residual < 1e-10 and sol.divergence_inf < 1e-10
