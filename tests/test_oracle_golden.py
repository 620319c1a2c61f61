"""The oracle against the reference's own outputs (golden fixtures).

Tolerances follow the reference's own tests: loop-vs-vectorised stencils at
1e-13 (``tests/core/test_kernels.py:33-41``), Tensor-vs-Direct Stokes at 3e-11
(``tests/core/test_stokes.py:37-51``), frozen scalar map at 2e-16
(``tests/core/test_scalar_correction.py:10-28``).  The oracle and the reference
run the same SciPy transforms and CG, so most checks are far tighter.
"""
import numpy as np
import pytest

import oracle as O
from helpers import golden


def _grid(shape):
    nx, ny, lx, ly = shape
    return O.Grid(int(nx), int(ny), float(lx), float(ly))


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_operators_match_reference(tag):
    d = golden("operators")
    g = _grid(d[f"{tag}_shape"])
    x, p = d[f"{tag}_x"], d[f"{tag}_p"]
    np.testing.assert_allclose(O.apply_K(g, x), d[f"{tag}_Kx"], rtol=1e-13, atol=1e-13 * np.abs(d[f"{tag}_Kx"]).max())
    np.testing.assert_allclose(O.apply_D(g, x), d[f"{tag}_Dx"], atol=1e-12)
    np.testing.assert_allclose(O.apply_D(g, x), d[f"{tag}_Dx_loop"], atol=1e-12)
    np.testing.assert_allclose(O.apply_Dt(g, p), d[f"{tag}_Dtp"], atol=1e-12)
    np.testing.assert_allclose(O.apply_Dt(g, p), d[f"{tag}_Dtp_loop"], atol=1e-12)
    np.testing.assert_allclose(O.nonlinear(g, x), d[f"{tag}_conv"], rtol=1e-13,
                               atol=1e-13 * np.abs(d[f"{tag}_conv"]).max())


def test_D_is_adjoint_and_annihilates_curl():
    g = O.Grid(9, 7, 1.3, .8)
    rng = np.random.default_rng(1)
    x, p = rng.standard_normal(g.size), rng.standard_normal(g.np)
    assert abs(np.dot(O.apply_D(g, x), p) - np.dot(x, O.apply_Dt(g, p))) < 1e-10
    np.testing.assert_array_equal(O.apply_Dt(g, np.ones(g.np)), np.zeros(g.size))
    psi = rng.standard_normal((g.ny + 1, g.nx + 1))
    psi[[0, -1], :] = 0
    psi[:, [0, -1]] = 0
    u, v = np.diff(psi, axis=0) / g.hy, -np.diff(psi, axis=1) / g.hx
    np.testing.assert_allclose(O.apply_D(g, g.pack(u, v)), 0.0, atol=1e-12)


@pytest.mark.parametrize("name", ["stokes_7x5", "stokes_11x7", "stokes_64"])
def test_tensor_stokes_matches_reference(name):
    d = golden(name)
    g = _grid(d["shape"])
    tol = 1e-9 if name == "stokes_64" else 1e-10
    solver = O.TensorStokesOracle(g, tolerance=tol, krylov_tolerance=1e-12)
    for k, (m, kappa) in enumerate(d["shifts"]):
        r = solver.solve(d["rhs"], mass=float(m), viscosity=float(kappa))
        scale = max(1.0, np.abs(d[f"vel{k}"]).max())
        np.testing.assert_allclose(r.velocity, d[f"vel{k}"], atol=1e-12 * scale)
        np.testing.assert_allclose(r.pressure, d[f"pres{k}"], atol=1e-12 * max(1.0, np.abs(d[f"pres{k}"]).max()))
        assert tuple(solver.last_iterations) == tuple(d[f"iters{k}"])
        assert r.residual <= tol and abs(r.residual - float(d[f"residual{k}"])) < 1e-12
        assert abs(r.divergence_inf - float(d[f"divergence{k}"])) < 1e-10


def test_scalar_correction_matches_reference():
    d = golden("scalar")
    for case, out in zip(d["cases"], d["outs"]):
        order, pred, dt, dd, rhs, alpha, beta = case
        r = O.solve_scalar_stage(pred, dt, dd, rhs, alpha, beta, order=int(order))
        np.testing.assert_allclose([r.values[0], r.values[-1], r.factor, r.coupling, len(r.values)], out,
                                   atol=2e-16, rtol=0)


@pytest.mark.parametrize("name", ["sdirk2_mrsav", "sdirk3_mrsav", "sdirk2", "sdirk3", "imex_euler",
                                  "imex_euler_mrsav"])
def test_one_step_matches_reference(name):
    d = golden(f"step_{name}")
    g = _grid(d["shape"])
    model = O.OracleModel(g, float(d["nu"]), backend=O.TensorStokesOracle(g, 1e-9, 1e-12))
    state = model.state(float(d["t0"]), d["x0"], float(d["r0"]))
    trial = O.make_scheme(name, gamma=float(d["gamma"])).step(model, state, float(d["dt"]))
    np.testing.assert_allclose(model.vector(trial.state), d["x1"], atol=1e-12 * np.abs(d["x1"]).max())
    assert abs(trial.state.r - float(d["r1"])) < 1e-13
    assert trial.state.t == float(d["t1"])
    if d["embedded"].size:
        np.testing.assert_allclose(trial.embedded_velocity, d["embedded"], atol=1e-11 * np.abs(d["embedded"]).max())
    for k, s in enumerate(trial.stages):
        ref = d[f"stage{k}"]
        got = np.array([s.r, s.residual, s.scalar_residual, s.divergence_inf, s.continuity_residual,
                        s.correction_predictor, s.frozen_factor] + list(s.corrections)
                       + [np.nan] * (2 - len(s.corrections)))
        np.testing.assert_allclose(got[[0, 5, 6, 7, 8]], ref[[0, 5, 6, 7, 8]], atol=1e-13)
        # residual-type fields are rounding-level numbers: same order of magnitude
        for i in (1, 2, 3):
            assert got[i] < 1e-8 and ref[i] < 1e-8
        np.testing.assert_allclose(s.pressure, d[f"stage{k}_pressure"],
                                   atol=1e-10 * max(1.0, np.abs(d[f"stage{k}_pressure"]).max()))


def test_config1_trajectory_matches_reference():
    d = golden("config1_64")
    g = O.Grid(64, 64)
    model = O.OracleModel(g, 1e-2, backend=O.TensorStokesOracle(g, 1e-9, 1e-12))
    steps = int(d["steps"])
    res = O.integrate(model, O.make_scheme("sdirk2_mrsav"), model.state(0.0, d["x0"], 0.0), [1e-3] * steps)
    assert res.status == "complete", res.error
    xf = model.vector(res.final)
    rel = np.linalg.norm(xf - d["x_final"]) / np.linalg.norm(d["x_final"])
    assert rel < 1e-11
    assert abs(res.final.r - float(d["r_final"])) < 1e-12
    keys = [str(k) for k in d["diag_keys"]]
    got = np.array([[row[k] for k in keys] for row in res.diagnostics])
    np.testing.assert_allclose(got, d["diagnostics"], rtol=1e-10, atol=1e-12)
    assert model.backend.total_iterations == int(d["iterations"])
