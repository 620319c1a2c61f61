"""CUDA operators, transforms and the FP64 Stokes solve against the reference.

Every call goes through the C ABI (include/macsav.h) via ctypes.  Bars: the
stencils at 1e-13 relative (the reference's own loop-vs-vectorised bar,
tests/core/test_kernels.py:33-41), transforms at 1e-13 against scipy.fft, the
Stokes solve at <= 1e-11 relative L2 with identical CG iteration counts.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import golden, load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    pkg = load_package()
    from importlib import import_module
    stokes = import_module(pkg.__name__ + ".stokes")
    lib = import_module(pkg.__name__ + "._lib")
    return pkg, stokes, lib, torch


def _plan(env, nx, ny, lx, ly):
    pkg, stokes, lib, torch = env
    return stokes.Plan(pkg.MACGrid(int(nx), int(ny), float(lx), float(ly)))


def _call(env, plan, fn, x, out_len, cols=1):
    pkg, stokes, lib, torch = env
    xd = torch.as_tensor(np.ascontiguousarray(x), device="cuda")
    out = torch.empty(out_len * cols, dtype=torch.float64, device="cuda")
    plan.check(getattr(plan.lib, fn)(plan.handle, stokes.dptr(xd), stokes.dptr(out), cols, stokes.stream_handle()))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_stencils_match_reference(env, tag):
    d = golden("operators")
    nx, ny, lx, ly = d[f"{tag}_shape"]
    g = O.Grid(int(nx), int(ny), float(lx), float(ly))
    plan = _plan(env, nx, ny, lx, ly)
    x, p = d[f"{tag}_x"], d[f"{tag}_p"]
    Kx = _call(env, plan, "macsav_apply_K", x, g.size)
    np.testing.assert_allclose(Kx, d[f"{tag}_Kx"], rtol=1e-13, atol=1e-13 * np.abs(d[f"{tag}_Kx"]).max())
    np.testing.assert_allclose(_call(env, plan, "macsav_apply_D", x, g.np), d[f"{tag}_Dx"], atol=1e-12)
    # two columns, column-blocked
    Dtp = _call(env, plan, "macsav_apply_Dt", np.ascontiguousarray(p.T).ravel(), g.size, cols=2)
    np.testing.assert_allclose(Dtp.reshape(2, -1).T, d[f"{tag}_Dtp"], atol=1e-12)
    conv = _call(env, plan, "macsav_convection", x, g.size)
    np.testing.assert_allclose(conv, d[f"{tag}_conv"], rtol=1e-13, atol=1e-13 * np.abs(d[f"{tag}_conv"]).max())


@pytest.mark.parametrize("kind,name", [(0, "dct2"), (1, "dst2"), (2, "dst1")])
@pytest.mark.parametrize("n", [2, 3, 5, 7, 8, 12, 63, 64, 96, 127, 255, 256, 1023, 1024, 2047])
def test_transforms_match_scipy(env, kind, name, n):
    pkg, stokes, lib, torch = env
    plan = _plan(env, 8, 8, 1.0, 1.0)
    rows = 5
    a = np.random.default_rng(n + 7 * kind).normal(size=(rows, n))
    ad = torch.as_tensor(a, device="cuda")
    out = torch.empty_like(ad)
    for inverse in (0, 1):
        plan.check(plan.lib.macsav_transform(plan.handle, kind, inverse, rows, n, stokes.dptr(ad),
                                             stokes.dptr(out), stokes.stream_handle()))
        torch.cuda.synchronize()
        ref = O.trig_transform(a, name, 1, bool(inverse))
        np.testing.assert_allclose(out.cpu().numpy(), ref, atol=1e-13 * max(1.0, np.abs(ref).max()) * np.log2(n + 2))


@pytest.mark.parametrize("name", ["stokes_7x5", "stokes_11x7", "stokes_64"])
def test_stokes_fp64_matches_reference(env, name):
    pkg, stokes, lib, torch = env
    d = golden(name)
    nx, ny, lx, ly = d["shape"]
    tol = 1e-9 if name == "stokes_64" else 1e-10
    solver = stokes.TensorStokes(pkg.MACGrid(int(nx), int(ny), float(lx), float(ly)), tolerance=tol,
                                 krylov_tolerance=1e-12)
    for k, (m, kappa) in enumerate(d["shifts"]):
        r = solver.solve(d["rhs"], mass=float(m), viscosity=float(kappa))
        for got, ref in ((r.velocity, d[f"vel{k}"]), (r.pressure, d[f"pres{k}"])):
            rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)
            assert rel <= 1e-11, (name, k, rel)
        assert solver.last_iterations == tuple(int(i) for i in d[f"iters{k}"])
        assert r.residual <= tol and r.divergence_inf <= tol * (1 + np.abs(r.velocity).max())
        assert abs(r.pressure.mean(axis=(0, 1))).max() < 1e-12


def test_stokes_single_column_and_gradient_rhs(env):
    """Gradient RHS gives zero velocity and recovers the pressure
    (tests/core/test_stokes.py:54-68, rectangle and three shifts)."""
    pkg, stokes, lib, torch = env
    g = O.Grid(8, 6)
    rng = np.random.default_rng(23)
    p = rng.normal(size=g.np)
    p -= p.mean()
    solver = stokes.TensorStokes(pkg.MACGrid(8, 6), tolerance=1e-10)
    for visc in (0.02, 0.05, 0.11):
        r = solver.solve(-O.apply_Dt(g, p), mass=1.0, viscosity=visc)
        np.testing.assert_allclose(r.velocity, 0.0, atol=2e-11)
        np.testing.assert_allclose(r.pressure.ravel(), p, atol=2e-10)
    assert solver.solves == 3 and solver.total_iterations > 0


def test_stokes_errors_match_reference(env):
    pkg, stokes, lib, torch = env
    g = pkg.MACGrid(7, 5, 2.0, 1.0)
    solver = stokes.TensorStokes(g, tolerance=1e-10)
    rhs = np.random.default_rng(1).normal(size=g.size)
    with pytest.raises(ValueError, match="Require mass,viscosity"):
        solver.solve(rhs, mass=-1.0, viscosity=0.1)
    with pytest.raises(ValueError, match="Require mass,viscosity"):
        solver.solve(rhs, mass=0.0, viscosity=0.0)
    bad = rhs.copy()
    bad[3] = np.nan
    with pytest.raises(ValueError, match="Invalid Stokes RHS"):
        solver.solve(bad, mass=1.0, viscosity=0.1)
    with pytest.raises(ValueError, match="Invalid Stokes RHS"):
        solver.solve(rhs[:-1], mass=1.0, viscosity=0.1)
    one = stokes.TensorStokes(g, tolerance=1e-10, max_iterations=1)
    with pytest.raises(RuntimeError, match=r"Pressure Schur CG failed with info=1"):
        one.solve(rhs, mass=1.0, viscosity=0.1)
    tight = stokes.TensorStokes(g, tolerance=1e-30)
    with pytest.raises(RuntimeError, match=r"Stokes residual=.*divergence="):
        tight.solve(rhs, mass=1.0, viscosity=0.1)


def test_zero_rhs_column(env):
    pkg, stokes, lib, torch = env
    g = pkg.MACGrid(9, 7)
    rhs = np.zeros((g.size, 2))
    rhs[:, 1] = np.random.default_rng(3).normal(size=g.size)
    solver = stokes.TensorStokes(g, tolerance=1e-10)
    r = solver.solve(rhs, mass=1.0, viscosity=0.05)
    assert solver.last_iterations[0] == 0 and solver.last_iterations[1] > 0
    assert np.all(r.velocity[:, 0] == 0) and np.all(r.pressure[:, :, 0] == 0)


def test_rhs_untouched_and_deterministic(env):
    pkg, stokes, lib, torch = env
    g = pkg.MACGrid(64, 48, 4 / 3, 1.0)
    rhs = np.random.default_rng(43).normal(size=(g.size, 2))
    orig = rhs.copy()
    solver = stokes.TensorStokes(g, tolerance=1e-9)
    a = solver.solve(rhs, mass=1.0, viscosity=1e-3)
    b = solver.solve(rhs, mass=1.0, viscosity=1e-3)
    np.testing.assert_array_equal(rhs, orig)
    np.testing.assert_array_equal(a.velocity, b.velocity)
    np.testing.assert_array_equal(a.pressure, b.pressure)


def test_diagnostics_and_reductions(env):
    pkg, stokes, lib, torch = env
    g = O.Grid(11, 7, 2.0, .7)
    x = np.random.default_rng(5).normal(size=g.size)
    f = np.random.default_rng(6).normal(size=g.size)
    plan = _plan(env, 11, 7, 2.0, .7)
    xd, fd = torch.as_tensor(x, device="cuda"), torch.as_tensor(f, device="cuda")
    out = (C.c_double * 8)()
    plan.check(plan.lib.macsav_diagnostics(plan.handle, stokes.dptr(xd), 0.3, 0.05, stokes.dptr(fd), out,
                                           stokes.stream_handle()))
    model = O.OracleModel(g, 0.05, force=lambda t: f)
    ref = model.diagnostics(O.State(0.0, *g.unpack(x), 0.3))
    keys = ["kinetic", "modified_energy", "divergence_inf", "h1_seminorm_squared", "r", "angular_momentum",
            "power", "dissipation"]
    np.testing.assert_allclose(list(out), [ref[k] for k in keys], rtol=1e-12, atol=1e-13)
    res = C.c_double()
    plan.check(plan.lib.macsav_inner(plan.handle, stokes.dptr(xd), stokes.dptr(fd), g.size, C.byref(res),
                                     stokes.stream_handle()))
    assert abs(res.value - g.inner(x, f)) < 1e-12 * abs(g.inner(x, f)) + 1e-14
    plan.check(plan.lib.macsav_max_abs(plan.handle, stokes.dptr(xd), g.size, C.byref(res), stokes.stream_handle()))
    assert res.value == np.abs(x).max()


@pytest.mark.parametrize("name", ["stokes_7x5", "stokes_11x7", "stokes_64"])
def test_stokes_fp32_mixed_meets_gates_and_matches(env, name):
    """FP32 transforms + FP64 defect correction: same gates as the reference,
    within 1e-9 relative L2 of the reference's FP64 solution."""
    pkg, stokes, lib, torch = env
    d = golden(name)
    nx, ny, lx, ly = d["shape"]
    tol = 1e-9 if name == "stokes_64" else 1e-10
    solver = stokes.TensorStokes(pkg.MACGrid(int(nx), int(ny), float(lx), float(ly)), tolerance=tol,
                                 krylov_tolerance=1e-12, precision="fp32")
    for k, (m, kappa) in enumerate(d["shifts"]):
        r = solver.solve(d["rhs"], mass=float(m), viscosity=float(kappa))
        for got, ref in ((r.velocity, d[f"vel{k}"]), (r.pressure, d[f"pres{k}"])):
            rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)
            assert rel <= 1e-9, (name, k, rel)
        assert r.residual <= tol and r.divergence_inf <= tol * (1 + np.abs(r.velocity).max())
        assert solver.last_refinements >= 1


@pytest.mark.parametrize("shape", [(256, 128, 2.0, 1.0), (512, 64, 8.0, 1.0), (96, 192, 0.5, 1.0),
                                   (1024, 32, 32.0, 1.0)])
def test_stokes_power_of_two_kernels_match_oracle(env, shape):
    """Larger grids exercise the compile-time-length FFT kernels (L = 64..2048)
    and the runtime-radix fallback (96, 192); checked against the oracle."""
    pkg, stokes, lib, torch = env
    nx, ny, lx, ly = shape
    og = O.Grid(nx, ny, lx, ly)
    rng = np.random.default_rng(nx + ny)
    rhs = rng.normal(size=(og.size, 2))
    ref = O.TensorStokesOracle(og, 1e-9, 1e-12).solve(rhs, mass=1.0, viscosity=3e-4)
    for precision, bar in (("fp64", 1e-11), ("fp32", 1e-9)):
        solver = stokes.TensorStokes(pkg.MACGrid(nx, ny, lx, ly), tolerance=1e-9, precision=precision)
        got = solver.solve(rhs, mass=1.0, viscosity=3e-4)
        for a, b in ((got.velocity, ref.velocity), (got.pressure, ref.pressure)):
            assert np.linalg.norm(a - b) / np.linalg.norm(b) < bar, precision
