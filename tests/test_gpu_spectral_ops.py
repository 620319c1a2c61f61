"""The Stokes solve's two spectral operators on their own, through the C ABI,
against the oracle (solver/mac/tensor_stokes.py:200-243,281-287):

* ``velocity_inverse``: (m I + k K)^{-1} of packed velocities, the u block's
  DST-I x DST-II and the v block's DST-II x DST-I transforms;
* ``precondition``: m (D D^T)^+ p + k p on the mean-zero part, DCT-II x DCT-II.

Sizes: the full-size grids of the workloads (512^2, 1024^2, 2048 x 1024:
the compile-time-length passes) and small or odd grids that take the
mixed-radix and direct-DFT passes (64 x 48, 96 x 192, 9 x 7).  Inputs: two
columns, white noise and the seeded curl field.

Bars (relative L2 per block against the oracle in FP64): FP64 1e-12, FP32
2e-6 (the FP32 FFT class; these operators are the inner solves' under the
FP64-accurate defect correction, which sets the accuracy of the Stokes
solution).
"""
import numpy as np
import pytest

import oracle as O
from helpers import load_package

pytestmark = pytest.mark.gpu

SHAPES = [(512, 512, 1.0, 1.0), (1024, 1024, 1.0, 1.0), (2048, 1024, 2.0, 1.0), (64, 48, 1.0, 0.75),
          (96, 192, 1.0, 2.0), (9, 7, 1.0, 1.0)]


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(b))


def _fields(pkg, og, nx, ny, lx, ly, n, seed):
    rng = np.random.default_rng(seed)
    curl = pkg.fields.packed_curl_velocity(nx, ny, lx, ly, min(8, nx // 4, ny // 4) or 1, seed)
    if n == og.size:
        return np.column_stack([rng.normal(size=n), curl])
    cells = rng.normal(size=(n, 2))
    cells[:, 1] += np.cos(np.pi * np.arange(n) / n)
    return cells


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: f"{s[0]}x{s[1]}")
def test_velocity_inverse_and_preconditioner_match_oracle(pkg, shape):
    nx, ny, lx, ly = shape
    og = O.Grid(nx, ny, lx, ly)
    g = pkg.MACGrid(nx, ny, lx, ly)
    ref_solver = O.TensorStokesOracle(og, 1e-9, 1e-12)
    from importlib import import_module
    stokes = import_module(pkg.__name__ + ".stokes")
    vel_in = _fields(pkg, og, nx, ny, lx, ly, og.size, 7)
    p_in = _fields(pkg, og, nx, ny, lx, ly, og.np, 8)
    for mass, visc in ((1.0, 2.5e-9), (1.0, 0.05 * og.hx * og.hy), (0.0, 1.0)):
        ref_u = ref_solver.velocity_inverse(vel_in, mass, visc)
        pm = p_in - p_in.mean(axis=0)
        ref_p = mass * ref_solver.poisson_inverse(pm) + visc * pm
        ref_p -= ref_p.mean(axis=0)
        for precision in ("fp64", "fp32"):
            solver = stokes.TensorStokes(g, precision=precision)
            got_u = solver.velocity_inverse(vel_in, mass, visc)
            got_p = solver.precondition(p_in, mass, visc)
            nu = og.n_u
            bar = 1e-12 if precision == "fp64" else 2e-6
            errs = (_rel(got_u[:nu], ref_u[:nu]), _rel(got_u[nu:], ref_u[nu:]), _rel(got_p, ref_p))
            assert max(errs) <= bar, (precision, mass, visc, errs)
            mean_bar = 1e-12 if precision == "fp64" else 1e-6
            assert np.abs(got_p.mean(axis=0)).max() <= mean_bar * np.abs(got_p).max()


def test_spectral_ops_reject_bad_shifts_and_columns(pkg):
    from importlib import import_module
    stokes = import_module(pkg.__name__ + ".stokes")
    g = pkg.MACGrid(16, 16)
    solver = stokes.TensorStokes(g, precision="fp32")
    x = np.ones(g.size)
    for mass, visc in ((-1.0, 1.0), (0.0, 0.0), (np.nan, 1.0)):
        with pytest.raises(ValueError):
            solver.velocity_inverse(x, mass, visc)
    with pytest.raises(ValueError):
        solver.precondition(np.ones((g.np, 5)), 1.0, 0.0)
    with pytest.raises(ValueError):
        solver.velocity_inverse(np.ones(g.size + 1), 1.0, 0.0)


@pytest.mark.parametrize("shape", [(512, 512, 1.0, 1.0), (1024, 1024, 1.0, 1.0), (2048, 1024, 2.0, 1.0)],
                         ids=lambda s: f"{s[0]}x{s[1]}")
def test_launch_shapes_give_the_same_bits(pkg, shape):
    """Every launch shape of the FP32 transform passes (one butterfly per
    thread, doubled threads, split lines: macsav_plan_set_launch_shape)
    computes each butterfly with the same arithmetic, so the operators and a
    whole FP32-bulk Stokes solve are bitwise equal across shapes."""
    nx, ny, lx, ly = shape
    og = O.Grid(nx, ny, lx, ly)
    g = pkg.MACGrid(nx, ny, lx, ly)
    from importlib import import_module
    stokes = import_module(pkg.__name__ + ".stokes")
    vel_in = _fields(pkg, og, nx, ny, lx, ly, og.size, 3)
    p_in = _fields(pkg, og, nx, ny, lx, ly, og.np, 4)
    solver = stokes.TensorStokes(g, precision="fp32")
    outs = []
    for s in (0, 1, 2, 3):
        solver.plan.check(solver.plan.lib.macsav_plan_set_launch_shape(solver.plan.handle, s))
        res = solver.solve(vel_in, mass=1.0, viscosity=1e-4 * 0.25)
        outs.append((solver.velocity_inverse(vel_in, 1.0, 2.5e-9), solver.precondition(p_in, 1.0, 2.5e-9),
                     res.velocity, res.pressure, solver.last_iterations))
    for s in (1, 2, 3):
        for a, b in zip(outs[0], outs[s]):
            np.testing.assert_array_equal(np.asarray(a), np.asarray(b))
    with pytest.raises(Exception):
        solver.plan.check(solver.plan.lib.macsav_plan_set_launch_shape(solver.plan.handle, 4))


def test_launch_shape_autotuner_keeps_the_bits(pkg):
    """The autotuner (macsav_plan_autotune_launch_shapes) only picks among
    shapes that compute the same bits: a solve before and after it agrees
    bitwise; plans tune only when asked."""
    nx = ny = 512
    og = O.Grid(nx, ny, 1.0, 1.0)
    g = pkg.MACGrid(nx, ny, 1.0, 1.0)
    from importlib import import_module
    stokes = import_module(pkg.__name__ + ".stokes")
    rhs = _fields(pkg, og, nx, ny, 1.0, 1.0, og.size, 5)
    plain = stokes.TensorStokes(g, precision="fp32")
    assert plain.plan.launch_shapes is None
    tuned = stokes.TensorStokes(g, precision="fp32", autotune_launch_shapes=True)
    assert set(tuned.plan.launch_shapes) == set(stokes.SHAPE_KINDS)
    assert set(tuned.plan.launch_shapes.values()) <= set(stokes.SHAPE_NAMES)
    a = plain.solve(rhs, mass=1.0, viscosity=2.5e-5)
    b = tuned.solve(rhs, mass=1.0, viscosity=2.5e-5)
    np.testing.assert_array_equal(a.velocity, b.velocity)
    np.testing.assert_array_equal(a.pressure, b.pressure)
    assert plain.last_iterations == tuned.last_iterations
    again = tuned.plan.autotune_launch_shapes(reps=5)
    assert set(again) == set(stokes.SHAPE_KINDS)
    np.testing.assert_array_equal(tuned.solve(rhs, mass=1.0, viscosity=2.5e-5).velocity, a.velocity)
    with pytest.raises(Exception):
        stokes.TensorStokes(pkg.MACGrid(64, 64), precision="fp64").plan.autotune_launch_shapes()
