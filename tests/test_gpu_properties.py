"""Behavioural properties that the reference's own tests check, run on the GPU path.

Each test restates one reference test (file:line in its docstring) against the
fused device schemes and the device TensorStokes: the zero-velocity closed form
of the SAV scalar, Laplacian reuse per stage, the discrete SAV energy balance,
preservation of a steady state, second/third order in time against an exact
semidiscrete solution, second order in space of the Stokes solve on a
manufactured solution, and the scalar-map and stage-gate failures with the
reference's exception types and messages.  The bars are the reference's.
"""
import re

import numpy as np
import pytest

import oracle as O
from helpers import load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def vortex(g, amplitude):
    """Discrete curl of the vertex stream function a sin^2(pi x/lx) sin^2(pi y/ly)
    (exactly divergence free on the MAC grid), as in tests/references/mac.py:14-21."""
    x, y = g.coordinates("vertex")
    psi = amplitude * np.sin(np.pi * x / g.lx) ** 2 * np.sin(np.pi * y / g.ly) ** 2
    psi[[0, -1], :] = 0
    psi[:, [0, -1]] = 0
    return g.pack(np.diff(psi, axis=0) / g.hy, -np.diff(psi, axis=1) / g.hx)


def manufactured(g, nu, amplitude):
    """Steady Stokes solution u = curl(sin^2 sin^2), p = cos cos and its load
    -nu lap u + grad p at the faces (the steady case of
    tests/references/mac.py:23-54, derivatives written out by hand)."""
    ax, ay = np.pi / g.lx, np.pi / g.ly
    xu, yu = g.coordinates("u")
    xv, yv = g.coordinates("v")
    xp, yp = g.coordinates("p")
    sx2u = np.sin(ax * xu) ** 2
    u = ay * sx2u * np.sin(2 * ay * yu)
    lap_u = ay * np.sin(2 * ay * yu) * (2 * ax ** 2 * np.cos(2 * ax * xu) - 4 * ay ** 2 * sx2u)
    fu = -nu * lap_u - ax * np.sin(ax * xu) * np.cos(ay * yu)
    sy2v = np.sin(ay * yv) ** 2
    v = -ax * np.sin(2 * ax * xv) * sy2v
    lap_v = -ax * np.sin(2 * ax * xv) * (2 * ay ** 2 * np.cos(2 * ay * yv) - 4 * ax ** 2 * sy2v)
    fv = -nu * lap_v - ay * np.cos(ax * xv) * np.sin(ay * yv)
    for a in (u, fu):
        a[:, [0, -1]] = 0
    for a in (v, fv):
        a[[0, -1], :] = 0
    p = np.cos(ax * xp) * np.cos(ay * yp)
    p -= p.mean()
    return amplitude * g.pack(u, v), amplitude * p, amplitude * g.pack(fu, fv)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("name", ["sdirk2", "sdirk2_mrsav"])
def test_zero_velocity_and_scalar_decay(pkg, name, graph):
    """tests/core/test_schemes.py:11-24: zero velocity stays zero and the SAV
    scalar follows the closed form of the two frozen-factor stages."""
    g = pkg.MACGrid(6, 4)
    model = pkg.MACNavierStokes(g, 0.1, use_graph=graph)
    trial = pkg.make_scheme(name, 2.0).step(model, model.state(0.0, np.zeros(g.size), 0.3), 0.03)
    assert np.linalg.norm(trial.state.u) < 1e-14
    assert np.linalg.norm(trial.state.v) < 1e-14
    if name == "sdirk2_mrsav":
        eta = 1 - 1 / np.sqrt(2)
        expected = 0.3 * (1 - (1 - 2 * eta) * 2 * 0.03) / (1 + eta * 2 * 0.03) ** 2
        assert trial.state.r == pytest.approx(expected, rel=1e-14)
        assert max(s.scalar_residual for s in trial.stages) < 1e-12


@pytest.mark.parametrize(("name", "calls"), [("sdirk2", 1), ("sdirk2_mrsav", 2), ("sdirk3", 3), ("sdirk3_mrsav", 4)])
def test_each_stage_laplacian_is_reused(pkg, name, calls):
    """tests/core/test_schemes.py:28-52: scheme code written against the model
    seam calls apply_K once per implicit stage on the device model, and its
    step equals the fused device step."""
    g = pkg.MACGrid(6, 4)
    model = pkg.MACNavierStokes(g, 0.1)
    original = model.apply_K
    count = [0]

    def counted(x):
        count[0] += 1
        return original(x)

    model.apply_K = counted
    x0 = pkg.fields.packed_curl_velocity(6, 4, 1.0, 1.0, 2, 3)
    seam = O.make_scheme(name).step(model, model.state(0.0, x0, 0.3), 0.03)
    assert count[0] == calls
    model.apply_K = original
    fused = pkg.make_scheme(name).step(model, model.state(0.0, x0, 0.3), 0.03)
    a, b = model.vector(seam.state), model.vector(fused.state)
    assert np.linalg.norm(a - b) <= 1e-12 * np.linalg.norm(b)
    assert seam.state.r == pytest.approx(fused.state.r, abs=1e-13)


@pytest.mark.parametrize("graph", [False, True])
def test_sav_discrete_energy_balance(pkg, graph):
    """tests/core/test_numerics.py:40-55: the two sdirk2_mrsav stages satisfy
    the discrete modified-energy identity to 1e-11."""
    og = O.Grid(10, 8)
    g = pkg.MACGrid(10, 8)
    model = pkg.MACNavierStokes(g, 0.03, use_graph=graph)
    old = vortex(og, 0.8)
    dt, r0, eta = 0.02, 0.05, 1 - 1 / np.sqrt(2)
    n0 = O.nonlinear(og, old)
    trial = pkg.make_scheme("sdirk2_mrsav", 2.0).step(model, model.state(0.0, old, r0), dt)
    s1, s2 = trial.stages
    first = np.asarray(model.backend.solve(old - dt * eta * (1 + r0) * (1 - s1.r) * n0, mass=1.0,
                                           viscosity=model.nu * eta * dt).velocity)
    second = model.vector(trial.state)
    velocities, scalars = [old, first, second], [r0, s1.r, s2.r]
    balance = 0.0
    for i in (1, 2):
        balance += og.inner(velocities[i] - velocities[i - 1], velocities[i]) \
            + (scalars[i] - scalars[i - 1]) * (scalars[i] - 1)
        for j in range(1, i + 1):
            a = eta if i == j else 1 - 2 * eta
            balance += dt * a * (model.nu * og.inner(O.apply_K(og, velocities[j]), velocities[i])
                                 + 2.0 * scalars[j] * (scalars[i] - 1))
    assert abs(balance) < 1e-11


@pytest.mark.parametrize("graph", [False, True])
def test_steady_velocity_and_zero_scalar_are_preserved(pkg, graph):
    """tests/core/test_sdirk3.py:24-37: a Stokes-solved velocity driven by
    its own steady load stays put under sdirk3 and sdirk3_mrsav."""
    g = pkg.MACGrid(8, 6)
    og = O.Grid(8, 6)
    model = pkg.MACNavierStokes(g, 0.1, use_graph=graph)
    drive = np.random.default_rng(7).normal(size=g.size)
    steady = np.asarray(model.backend.solve(drive, mass=1.0, viscosity=0.1).velocity)
    force = model.nu * O.apply_K(og, steady) + O.nonlinear(og, steady)
    model.force = lambda t: force
    state = model.state(0.0, steady)
    for name in ("sdirk3", "sdirk3_mrsav"):
        trial = pkg.make_scheme(name).step(model, state, 0.013)
        assert og.norm(model.vector(trial.state) - steady) < 1e-11
        assert abs(trial.state.r) < 1e-11


@pytest.mark.parametrize(("name", "horizon", "counts", "rate"), [
    ("sdirk2", 0.1, (10, 20, 40), 1.85), ("sdirk2_mrsav", 0.1, (10, 20, 40), 1.85),
    ("sdirk3", 1.0, (5, 10, 20), 2.85), ("sdirk3_mrsav", 1.0, (5, 10, 20), 2.85)])
def test_order_against_exact_semidiscrete_solution(pkg, name, horizon, counts, rate):
    """tests/core/test_numerics.py:25-38 (second order, T = 0.1) and the third
    order of tests/core/test_sdirk3.py:14-22, here on the MAC model with the
    forced exact solution exp(-t) u0 (T = 1)."""
    g = pkg.MACGrid(10, 8)
    og = O.Grid(10, 8)
    model = pkg.MACNavierStokes(g, 0.1, use_graph=True)
    base = vortex(og, 0.05)

    def force(t):
        z = np.exp(-t) * base
        return -z + model.nu * O.apply_K(og, z) + O.nonlinear(og, z)

    model.force = force
    errors = []
    for count in counts:
        result = pkg.run_fixed(model, pkg.make_scheme(name, 1.0), model.state(0.0, base), [horizon / count] * count)
        assert result.status == "complete", result.error
        errors.append(og.norm(model.vector(result.final) - np.exp(-horizon) * base))
    assert min(np.log2(np.array(errors[:-1]) / errors[1:])) > rate, errors


def test_stokes_spatial_convergence_and_operator_structure(pkg):
    """tests/core/test_numerics.py:11-23: K symmetric positive definite, and
    the device Stokes solve (mass 0) converges at second order in velocity
    and pressure on a rectangular domain."""
    errors = []
    for nx, ny in ((8, 6), (16, 12), (32, 24)):
        g = pkg.MACGrid(nx, ny, 1.3, 0.8)
        og = O.Grid(nx, ny, 1.3, 0.8)
        model = pkg.MACNavierStokes(g, 0.1)
        rng = np.random.default_rng(3)
        x, y = rng.normal(size=g.size), rng.normal(size=g.size)
        kx, ky = model.apply_K(x).cpu().numpy(), model.apply_K(y).cpu().numpy()
        assert abs(og.inner(kx, y) - og.inner(x, ky)) <= 1e-12 * abs(og.inner(kx, y))
        assert og.inner(x, kx) > 0
        exact, p, load = manufactured(og, 0.1, 0.1)
        solved = model.backend.solve(load, mass=0.0, viscosity=0.1)
        errors.append([og.norm(np.asarray(solved.velocity) - exact),
                       np.sqrt(og.area * np.sum((np.asarray(solved.pressure) - p) ** 2))])
    rates = np.log2(np.array(errors[:-1]) / np.array(errors[1:]))
    assert np.min(rates) > 1.7, (errors, rates)


def _oracle_error(name, g_args, nu, x0, t, r, dt, tol, ktol):
    og = O.Grid(*g_args)
    m = O.OracleModel(og, nu, backend=O.TensorStokesOracle(og, tol, ktol))
    try:
        O.make_scheme(name).step(m, m.state(t, x0, r), dt)
    except Exception as error:  # the reference's exception for this step
        return error
    return None


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize(("name", "r"), [("sdirk2_mrsav", float("nan")), ("sdirk3_mrsav", float("inf")),
                                         ("sdirk2_mrsav", 1e200), ("sdirk3_mrsav", -1e200),
                                         ("imex_euler_mrsav", float("nan"))])
def test_scalar_map_failures_raise_like_reference(pkg, name, r, graph):
    """scalar_correction.py:29-52 guards (inputs, denominator) and the IMEX
    Euler state check, raised with the reference's type and message."""
    x0 = pkg.fields.packed_curl_velocity(16, 12, 1.3, 0.8, 4, 3)
    want = _oracle_error(name, (16, 12, 1.3, 0.8), 0.05, x0, 0.1, r, 0.01, 1e-9, 1e-12)
    assert want is not None
    model = pkg.MACNavierStokes(pkg.MACGrid(16, 12, 1.3, 0.8), 0.05, use_graph=graph)
    with pytest.raises(type(want)) as got:
        pkg.make_scheme(name).step(model, model.state(0.1, x0, r), 0.01)
    assert str(got.value) == str(want)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("name", ["sdirk2_mrsav", "sdirk3_mrsav", "imex_euler_mrsav", "imex_euler"])
def test_stage_gate_failure_raises_like_reference(pkg, name, graph):
    """A Stokes backend loose enough to pass its own gate (1e-2) but not the
    stage gate (1e-8): the stage residual messages of sdirk2_mrsav.py:60-66,
    sdirk3_mrsav.py:105-114 and imex_euler*.py, with the same divergence."""
    x0 = pkg.fields.packed_curl_velocity(16, 12, 1.3, 0.8, 4, 3)
    want = _oracle_error(name, (16, 12, 1.3, 0.8), 0.05, x0, 0.1, 0.2, 0.01, 1e-2, 1e-6)
    assert isinstance(want, RuntimeError)
    backend = pkg.TensorStokes(pkg.MACGrid(16, 12, 1.3, 0.8), tolerance=1e-2, krylov_tolerance=1e-6)
    model = pkg.MACNavierStokes(pkg.MACGrid(16, 12, 1.3, 0.8), 0.05, backend=backend, use_graph=graph)
    with pytest.raises(RuntimeError) as got:
        pkg.make_scheme(name).step(model, model.state(0.1, x0, 0.2), 0.01)
    msg, ref = str(got.value), str(want)
    head = re.match(r"[A-Za-z ]+", ref).group(0)  # the text before the first number
    assert head.endswith("residuals ") or head.endswith("residual ")
    assert msg.startswith(head), (msg, ref)
    div = float(msg.rsplit(" ", 1)[1])
    assert div == pytest.approx(float(ref.rsplit(" ", 1)[1]), rel=1e-6)


FULL = [("cavity512", (512, 512, 1.0, 1.0), 1e-3, 2.5e-4, 16),
        ("cavity2048x1024", (2048, 1024, 2.0, 1.0), 5e-5, 1e-4, 64)]


@pytest.mark.parametrize(("shape", "nu", "dt", "modes"), [f[1:] for f in FULL], ids=[f[0] for f in FULL])
def test_full_size_fp32_bulk_tracks_fp64_and_gates_hold(pkg, shape, nu, dt, modes):
    """The single-cavity workloads at full size (512^2 and 2048 x 1024,
    sdirk3_mrsav, seeded curl fields): over two graph-captured steps every
    stage passes the reference's stage gates (solver/schemes/sdirk3_mrsav.py:
    18-65: residuals <= 1e-8, max |D u| <= 1e-8 (1 + max |u|)), and the
    FP32-bulk form stays within 1e-12 of the FP64 path in velocity and SAV
    scalar.  The last stage's pressures are compared through what they do to
    the velocity: dt |grad(p32 - p64)| <= 1e-9 |u| (the pressure enters the
    momentum balance only through its gradient, and with a weak pressure,
    norm 5e-4 here, its own relative difference is no measure)."""
    g = pkg.MACGrid(*shape)
    x0 = pkg.fields.packed_curl_velocity(shape[0], shape[1], shape[2], shape[3], modes, 20261203)
    out = {}
    for prec in ("fp64", "fp32"):
        model = pkg.MACNavierStokes(g, nu, precision=prec, use_graph=True)
        state = model.state(0.0, x0, 1.0)
        scheme = pkg.make_scheme("sdirk3_mrsav")
        for _ in range(2):
            trial = scheme.step(model, state, dt)
            state = trial.state
            umax = float(np.abs(model.vector(state)).max())
            for st in trial.stages:
                assert st.residual <= 1e-8 and st.scalar_residual <= 1e-8
                assert st.divergence_inf <= 1e-8 * (1.0 + umax)
        out[prec] = (model.vector(state), np.asarray(trial.stages[-1].pressure), state.r)
        del model
    (u64, p64, r64), (u32, p32, r32) = out["fp64"], out["fp32"]
    assert np.linalg.norm(u32 - u64) <= 1e-12 * np.linalg.norm(u64)
    dp = p32 - p64
    grad = np.sqrt(np.sum((np.diff(dp, axis=1) / g.hx) ** 2) + np.sum((np.diff(dp, axis=0) / g.hy) ** 2))
    assert dt * grad <= 1e-9 * np.linalg.norm(u64)
    assert abs(r32 - r64) <= 1e-12


def test_sav_discrete_energy_balance_at_512(pkg):
    """The discrete modified-energy identity of tests/core/test_numerics.py:40-55
    at the 512^2 workload size (sdirk2_mrsav, nu=1e-3, dt=2.5e-4); the bar is
    relative to the kinetic energy, as the identity's terms scale with it."""
    og = O.Grid(512, 512)
    g = pkg.MACGrid(512, 512)
    model = pkg.MACNavierStokes(g, 1e-3, use_graph=True)
    old = vortex(og, 0.8)
    dt, r0, eta = 2.5e-4, 0.9, 1 - 1 / np.sqrt(2)
    n0 = O.nonlinear(og, old)
    trial = pkg.make_scheme("sdirk2_mrsav", 2.0).step(model, model.state(0.0, old, r0), dt)
    s1, s2 = trial.stages
    first = np.asarray(model.backend.solve(old - dt * eta * (1 + r0) * (1 - s1.r) * n0, mass=1.0,
                                           viscosity=model.nu * eta * dt).velocity)
    second = model.vector(trial.state)
    velocities, scalars = [old, first, second], [r0, s1.r, s2.r]
    balance = 0.0
    for i in (1, 2):
        balance += og.inner(velocities[i] - velocities[i - 1], velocities[i]) \
            + (scalars[i] - scalars[i - 1]) * (scalars[i] - 1)
        for j in range(1, i + 1):
            a = eta if i == j else 1 - 2 * eta
            balance += dt * a * (model.nu * og.inner(O.apply_K(og, velocities[j]), velocities[i])
                                 + 2.0 * scalars[j] * (scalars[i] - 1))
    assert abs(balance) < 1e-11 * max(og.inner(old, old), 1.0)
