"""The fused device step and the GPU model seam against the reference (golden
fixtures) and the oracle, driven as a user drives them: one step at a time,
under the reference's fixed-step driver (its restatement in
oracle/integrate_oracle.py, since the reference cannot travel to the GPU
machine), and by the package's device-resident loop ``run_fixed``.

Bars: <= 1e-11 relative L2 on the stepped velocity and pressures (the parity
bar of the FP64 path), SAV scalars to 1e-12, identical CG iterations.
"""
import numpy as np
import pytest

import oracle as O
import oracle.integrate_oracle as DRV
from helpers import golden, load_package

pytestmark = pytest.mark.gpu
SCHEMES = ["sdirk2_mrsav", "sdirk3_mrsav", "sdirk2", "sdirk3", "imex_euler", "imex_euler_mrsav"]


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("name", SCHEMES)
def test_fused_step_matches_reference(pkg, name, graph):
    d = golden(f"step_{name}")
    nx, ny, lx, ly = d["shape"]
    g = pkg.MACGrid(int(nx), int(ny), float(lx), float(ly))
    model = pkg.MACNavierStokes(g, float(d["nu"]), use_graph=graph)
    state = model.state(float(d["t0"]), d["x0"], float(d["r0"]))
    scheme = pkg.make_scheme(name, gamma=float(d["gamma"]))
    for _ in range(2):  # second call replays the captured graph
        trial = scheme.step(model, state, float(d["dt"]))
    assert _rel(model.vector(trial.state), d["x1"]) < 1e-11
    assert abs(trial.state.r - float(d["r1"])) < 1e-12
    assert trial.state.t == float(d["t1"])
    if d["embedded"].size:
        assert _rel(trial.embedded_velocity.cpu().numpy(), d["embedded"]) < 1e-11
    for k, st in enumerate(trial.stages):
        ref = d[f"stage{k}"]
        assert abs(st.r - ref[0]) < 1e-12
        assert st.residual < 1e-8 and st.scalar_residual < 1e-8
        assert abs(st.divergence_inf - ref[3]) < 1e-9
        if "mrsav" in name:
            assert st.correction_predictor == pytest.approx(ref[5], abs=1e-12)
            assert st.frozen_factor == pytest.approx(ref[6], abs=1e-12)
            np.testing.assert_allclose(st.corrections, ref[7:7 + len(st.corrections)], atol=1e-12)
        assert _rel(np.asarray(st.pressure), d[f"stage{k}_pressure"]) < 1e-10


def test_config1_trajectory_matches_reference(pkg):
    """64^2, nu=1e-2, sdirk2_mrsav, dt=1e-3, 100 steps, psi modes <= 4."""
    d = golden("config1_64")
    g = pkg.MACGrid(64, 64)
    model = pkg.MACNavierStokes(g, 1e-2, use_graph=True)
    res = DRV.integrate(model, pkg.make_scheme("sdirk2_mrsav"), model.state(0.0, d["x0"], 0.0), [1e-3] * 100)
    assert res.status == "complete", res.error
    assert _rel(model.vector(res.final), d["x_final"]) < 1e-11
    assert abs(res.final.r - float(d["r_final"])) < 1e-12
    keys = [str(k) for k in d["diag_keys"]]
    got = np.array([[row[k] for k in keys] for row in res.diagnostics])
    np.testing.assert_allclose(got, d["diagnostics"], rtol=1e-10, atol=1e-12)
    # the package's device-resident loop over the same 100 steps
    fixed = pkg.run_fixed(model, pkg.make_scheme("sdirk2_mrsav"), model.state(0.0, d["x0"], 0.0), [1e-3] * 100)
    assert fixed.status == "complete" and len(fixed.times) == 101
    assert _rel(model.vector(fixed.final), d["x_final"]) < 1e-11
    assert abs(fixed.final.r - float(d["r_final"])) < 1e-12


def test_generic_scheme_code_runs_on_gpu_model(pkg):
    """The oracle's restated scheme classes (written against the model seam)
    drive the GPU model: Level-2 drop-in."""
    d = golden("step_sdirk3_mrsav")
    nx, ny, lx, ly = d["shape"]
    g = pkg.MACGrid(int(nx), int(ny), float(lx), float(ly))
    model = pkg.MACNavierStokes(g, float(d["nu"]))
    state = model.state(float(d["t0"]), d["x0"], float(d["r0"]))
    trial = O.SDIRK3MRSAV(float(d["gamma"])).step(model, state, float(d["dt"]))
    assert _rel(model.vector(trial.state), d["x1"]) < 1e-11
    assert abs(trial.state.r - float(d["r1"])) < 1e-12


def test_forced_step_matches_oracle(pkg):
    """Body force evaluated at the stage nodes (sdirk3.py:41)."""
    g = pkg.MACGrid(24, 16, 1.5, 1.0)
    og = O.Grid(24, 16, 1.5, 1.0)
    x0 = pkg.fields.packed_curl_velocity(24, 16, 1.5, 1.0, 4, 9)
    base = np.random.default_rng(4).normal(size=g.size)

    def force(t):
        return np.cos(3 * t) * base

    for name in ("sdirk3_mrsav", "sdirk2_mrsav", "sdirk3"):
        model = pkg.MACNavierStokes(g, 0.02, force=force)
        ref_model = O.OracleModel(og, 0.02, force=force, backend=O.TensorStokesOracle(og, 1e-9, 1e-12))
        trial = pkg.make_scheme(name).step(model, model.state(0.3, x0, 0.1), 0.004)
        ref = O.make_scheme(name).step(ref_model, ref_model.state(0.3, x0, 0.1), 0.004)
        assert _rel(model.vector(trial.state), ref_model.vector(ref.state)) < 1e-11
        assert abs(trial.state.r - ref.state.r) < 1e-12
        diag = model.diagnostics(trial.state)
        rdiag = ref_model.diagnostics(ref.state)
        for k in rdiag:
            assert diag[k] == pytest.approx(rdiag[k], rel=1e-9, abs=1e-12), k


def test_step_failure_is_reported_like_reference(pkg):
    """A NaN body force fails the step with the reference's exception and
    the reference's integrate keeps the accepted prefix (integrate.py:90-93)."""
    g = pkg.MACGrid(8, 6)
    model = pkg.MACNavierStokes(g, 0.1)
    x0 = pkg.fields.packed_curl_velocity(8, 6, 1.0, 1.0, 2, 1)
    calls = []

    def force(t):
        calls.append(t)
        return np.full(g.size, np.nan) if t > 0.012 else np.zeros(g.size)
    model.force = force
    res = DRV.integrate(model, pkg.make_scheme("sdirk2_mrsav"), model.state(0.0, x0), [0.01, 0.01, 0.01])
    assert res.status == "failed"
    assert res.error.startswith("ValueError: Invalid Stokes RHS")
    assert len(res.times) == 2
    # the device-resident loop: a failing stage check ends the run with its prefix
    backend = pkg.TensorStokes(g, max_iterations=1)
    bad = pkg.MACNavierStokes(g, 0.1, backend=backend)
    fixed = pkg.run_fixed(bad, pkg.make_scheme("sdirk2_mrsav"), bad.state(0.0, x0), [0.01, 0.01])
    assert fixed.status == "failed" and fixed.error.startswith("RuntimeError: Pressure Schur CG failed")
    assert fixed.times == [0.0] and fixed.final.t == 0.0


def test_cg_failure_inside_step(pkg):
    g = pkg.MACGrid(16, 12)
    backend = pkg.TensorStokes(g, max_iterations=1)
    model = pkg.MACNavierStokes(g, 0.05, backend=backend)
    x0 = pkg.fields.packed_curl_velocity(16, 12, 1.0, 1.0, 4, 2)
    with pytest.raises(RuntimeError, match=r"Pressure Schur CG failed with info=1"):
        pkg.make_scheme("sdirk3_mrsav").step(model, model.state(0.0, x0), 0.01)


@pytest.mark.parametrize("name", ["sdirk3_mrsav", "sdirk2_mrsav"])
def test_fp32_mixed_step_close_to_fp64(pkg, name):
    """The FP32-bulk step keeps the reference's gates and stays within 1e-9
    (far inside the 1e-6 budget) of the FP64 reference step."""
    d = golden(f"step_{name}")
    nx, ny, lx, ly = d["shape"]
    g = pkg.MACGrid(int(nx), int(ny), float(lx), float(ly))
    for graph in (False, True):
        model = pkg.MACNavierStokes(g, float(d["nu"]), precision="fp32", use_graph=graph)
        state = model.state(float(d["t0"]), d["x0"], float(d["r0"]))
        trial = pkg.make_scheme(name, gamma=float(d["gamma"])).step(model, state, float(d["dt"]))
        assert _rel(model.vector(trial.state), d["x1"]) < 1e-9
        assert abs(trial.state.r - float(d["r1"])) < 1e-10


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("name", ["sdirk3_mrsav", "sdirk2", "imex_euler"])
def test_embedded_norms_match_host_inner_products(pkg, name, graph):
    """The step's device inner products for the adaptive controller equal
    the model's own inner products of the returned fields."""
    d = golden("step_sdirk3_mrsav")
    nx, ny, lx, ly = d["shape"]
    g = pkg.MACGrid(int(nx), int(ny), float(lx), float(ly))
    model = pkg.MACNavierStokes(g, float(d["nu"]), use_graph=graph)
    state = model.state(0.1, d["x0"], 0.05)
    trial = pkg.make_scheme(name).step(model, state, 0.01)
    if trial.embedded_velocity is None:
        assert not hasattr(trial, "embedded_norms")
        return
    high = model.device_vector(trial.state)
    diff = model.combine((1.0, high), (-1.0, trial.embedded_velocity))
    expect = (model.inner(diff, diff), model.inner(state.device, state.device), model.inner(high, high))
    for got, want in zip(trial.embedded_norms[:3], expect):
        assert got == pytest.approx(want, rel=1e-12, abs=1e-300)
    assert trial.embedded_norms[3] == 0.0


def test_host_state_layout_over_mapped_pinned_memory(pkg):
    """The pinned host arrays of a State built by the model are read and
    written by the layout kernels directly; the result is bitwise the copy
    path's (MACGrid.pack / unpack, solver/mac/grid.py:52-65), pageable arrays
    take the copy path, and a step from either gives the same state."""
    import torch
    g = pkg.MACGrid(48, 40, 1.2, 1.0)
    model = pkg.MACNavierStokes(g, 1e-2)
    x = np.random.default_rng(7).standard_normal(g.size)
    st = model.state(0.0, x, 0.5)
    u_ref, v_ref = g.unpack(x)
    np.testing.assert_array_equal(st.u, u_ref)   # unpack: exact copies, zero walls
    np.testing.assert_array_equal(st.v, v_ref)
    assert isinstance(st.u.base, torch.Tensor) and st.u.base.is_pinned()
    mapped = model.device_vector(pkg.State(st.t, st.u, st.v, st.r))
    assert hasattr(mapped, "_host_faces")          # packed from the pinned arrays directly
    pageable = model.device_vector(pkg.State(st.t, np.array(st.u), np.array(st.v), st.r))
    assert not hasattr(pageable, "_host_faces")    # copied
    # writable pinned arrays are copied (blocking), so callers may reuse them at once
    writable = torch.from_numpy(np.array(st.u)).pin_memory().numpy()
    assert writable.flags.writeable
    copied = model.device_vector(pkg.State(st.t, writable, st.v, st.r))
    assert not hasattr(copied, "_host_faces")
    np.testing.assert_array_equal(mapped.cpu().numpy(), x)
    np.testing.assert_array_equal(pageable.cpu().numpy(), x)
    np.testing.assert_array_equal(copied.cpu().numpy(), x)
    scheme = pkg.make_scheme("sdirk2_mrsav")
    a = scheme.step(model, pkg.State(st.t, st.u, st.v, st.r), 1e-3).state
    b = scheme.step(model, pkg.State(st.t, np.array(st.u), np.array(st.v), st.r), 1e-3).state
    np.testing.assert_array_equal(a.u, b.u)
    np.testing.assert_array_equal(a.v, b.v)
    assert a.r == b.r
    # wall checks still apply to pinned arrays
    bad = model.state(0.0, x, 0.5)
    with pytest.raises(ValueError, match="Normal boundary velocities must be zero"):
        u_bad = torch.from_numpy(np.array(bad.u)).pin_memory()
        u_bad[0, 0] = 1.0
        model.device_vector(pkg.State(0.0, u_bad.numpy(), bad.v, 0.5))
