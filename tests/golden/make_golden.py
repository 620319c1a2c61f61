"""Generate the golden fixtures by running the reference itself.

Run from the repository root with the path of the reference's source tree,
given as the first argument or in the environment variable MACSAV_REFERENCE:

    python tests/golden/make_golden.py /path/to/reference

It imports the reference's own ``solver`` package (numba is absent, so the
identity ``njit`` stand-in from ``oracle/reference_shim`` is put first on the
path; bytecode writing is disabled so nothing is written into the reference
tree), runs the hot-path functions on seeded inputs and stores inputs and
outputs as ``tests/golden/*.npz``.  The fixtures are the pin for the oracle
(``tests/test_oracle_golden.py``) and a direct check for the CUDA path.
"""
from __future__ import annotations

import importlib.util
import json
import pathlib
import sys

import numpy as np

sys.dont_write_bytecode = True
HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parent.parent
_ref_arg = sys.argv[1] if len(sys.argv) > 1 else __import__("os").environ.get("MACSAV_REFERENCE")
if not _ref_arg:
    sys.exit("usage: make_golden.py REFERENCE_DIR (or set MACSAV_REFERENCE)")
REF = pathlib.Path(_ref_arg)
sys.path.insert(0, str(REPO / "oracle" / "reference_shim"))
sys.path.insert(0, str(REF))

from solver.mac.grid import MACGrid  # noqa: E402
from solver.mac.operators import MACOperators  # noqa: E402
from solver.mac import kernels  # noqa: E402
from solver.mac.tensor_stokes import TensorStokes  # noqa: E402
from solver.mac_ns import MACNavierStokes  # noqa: E402
from solver.schemes.registry import make_scheme  # noqa: E402
from solver.schemes.scalar_correction import solve_scalar_stage  # noqa: E402
from solver.integrate import integrate  # noqa: E402

_spec = importlib.util.spec_from_file_location("_fields", REPO / "mac-mr-sav-rk_gb300" / "fields.py")
fields = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(fields)


def save(name: str, **arrays) -> None:
    np.savez_compressed(HERE / f"{name}.npz", **{k: np.asarray(v) for k, v in arrays.items()})
    print("wrote", name, sum(np.asarray(v).nbytes for v in arrays.values()), "bytes raw")


def operators() -> None:
    """K, D, D^T (CSR and Numba loops) and convection on a rectangular grid."""
    out = {}
    for tag, (nx, ny, lx, ly) in {"a": (11, 7, 2.0, 0.7), "b": (9, 7, 1.3, 0.8), "c": (64, 48, 4 / 3, 1.0)}.items():
        g = MACGrid(nx, ny, lx, ly)
        ops = MACOperators(g)
        rng = np.random.default_rng(73 + nx)
        x = rng.normal(size=g.size)
        p = rng.normal(size=(g.np, 2))
        u, v = g.unpack(x)
        cu, cv = kernels.convection(u, v, g.hx, g.hy)
        out.update({f"{tag}_shape": [nx, ny, lx, ly], f"{tag}_x": x, f"{tag}_p": p,
                    f"{tag}_Kx": ops.K @ x, f"{tag}_Dx": ops.D @ x, f"{tag}_Dtp": ops.D.T @ p,
                    f"{tag}_Dx_loop": kernels.packed_divergence_vector(x, nx, ny, g.hx, g.hy),
                    f"{tag}_Dtp_loop": kernels.packed_divergence_transpose(p, nx, ny, g.hx, g.hy),
                    f"{tag}_conv": g.pack(cu, cv)})
    save("operators", **out)


def _stokes_case(nx, ny, lx, ly, rhs, shifts, tol=1e-10, ktol=1e-12):
    g = MACGrid(nx, ny, lx, ly)
    solver = TensorStokes(MACOperators(g), tolerance=tol, krylov_tolerance=ktol)
    res = {}
    for k, (m, kappa) in enumerate(shifts):
        r = solver.solve(rhs, mass=m, viscosity=kappa)
        res.update({f"vel{k}": r.velocity, f"pres{k}": r.pressure, f"residual{k}": r.residual,
                    f"divergence{k}": r.divergence_inf, f"iters{k}": np.array(solver.last_iterations)})
    return res


def stokes() -> None:
    """TensorStokes.solve on the reference tests' shapes and on a 64^2 stage-like RHS."""
    rhs = np.random.default_rng(19).normal(size=((7 - 1) * 5 + 7 * 4, 2))
    shifts = [(1.0, 0.07), (1.0, 0.0), (0.0, 0.07)]
    save("stokes_7x5", shape=[7, 5, 2.0, 1.0], rhs=rhs, shifts=shifts, **_stokes_case(7, 5, 2.0, 1.0, rhs, shifts))
    rhs = np.random.default_rng(37).normal(size=((11 - 1) * 7 + 11 * 6, 2))
    shifts = [(1.0, 0.03), (0.7, 0.09), (0.0, 0.05)]
    save("stokes_11x7", shape=[11, 7, 2.0, 1.0], rhs=rhs, shifts=shifts, **_stokes_case(11, 7, 2.0, 1.0, rhs, shifts))
    # 64^2 with a convection-like second column: the mr-SAV stage's two columns
    g = MACGrid(64, 64)
    x = fields.packed_curl_velocity(64, 64, 1.0, 1.0, 4, 1)
    u, v = g.unpack(x)
    cu, cv = kernels.convection(u, v, g.hx, g.hy)
    rhs = np.column_stack([x, g.pack(cu, cv)])
    shifts = [(1.0, 1e-2 * 1e-3 * (1 - 1 / np.sqrt(2))), (1.0, 1e-3)]
    save("stokes_64", shape=[64, 64, 1.0, 1.0], rhs=rhs, shifts=shifts, **_stokes_case(64, 64, 1.0, 1.0, rhs, shifts,
                                                                                       tol=1e-9))


def scalar() -> None:
    rng = np.random.default_rng(5)
    cases, outs = [], []
    for order in (1, 2, 3):
        for _ in range(6):
            pred, dt, d, rhs, alpha, beta = rng.normal(0, .5), rng.uniform(1e-4, .3), rng.uniform(1, 2), \
                rng.normal(0, .5), rng.normal(0, 2), rng.uniform(0, 3)
            r = solve_scalar_stage(pred, dt, d, rhs, alpha, beta, order=order)
            cases.append([order, pred, dt, d, rhs, alpha, beta])
            outs.append([r.values[0], r.values[-1], r.factor, r.coupling, len(r.values)])
    save("scalar", cases=np.array(cases), outs=np.array(outs))


def _stage_fields(trial):
    out = {}
    for k, s in enumerate(trial.stages):
        out[f"stage{k}"] = np.array([s.r, s.residual, s.scalar_residual, s.divergence_inf, s.continuity_residual,
                                     s.correction_predictor, s.frozen_factor] + list(s.corrections)
                                    + [np.nan] * (2 - len(s.corrections)))
        out[f"stage{k}_pressure"] = s.pressure
    return out


def schemes() -> None:
    """One step of every scheme from a seeded curl field on a rectangle."""
    g = MACGrid(16, 12, 1.3, 0.8)
    x0 = fields.packed_curl_velocity(16, 12, 1.3, 0.8, 4, 3)
    for name in ("sdirk2_mrsav", "sdirk3_mrsav", "sdirk2", "sdirk3", "imex_euler", "imex_euler_mrsav"):
        model = MACNavierStokes(g, 0.05)
        model.backend = TensorStokes(model.ops, tolerance=1e-9, krylov_tolerance=1e-12)
        state = model.state(0.1, x0, 0.05 if "mrsav" in name else 0.0)
        trial = make_scheme(name, gamma=1.5).step(model, state, 0.01)
        emb = trial.embedded_velocity
        save(f"step_{name}", shape=[16, 12, 1.3, 0.8], x0=x0, nu=0.05, t0=0.1, r0=state.r, dt=0.01, gamma=1.5,
             x1=model.vector(trial.state), r1=trial.state.r, t1=trial.state.t,
             embedded=(np.zeros(0) if emb is None else emb), **_stage_fields(trial))


def config1(steps: int = 100) -> None:
    """64^2, nu=1e-2, sdirk2_mrsav, dt=1e-3, psi modes k,l<=4, Krylov 1e-12."""
    g = MACGrid(64, 64)
    model = MACNavierStokes(g, 1e-2)
    model.backend = TensorStokes(model.ops, tolerance=1e-9, krylov_tolerance=1e-12)
    x0 = fields.packed_curl_velocity(64, 64, 1.0, 1.0, 4, 2024)
    res = integrate(model, make_scheme("sdirk2_mrsav"), model.state(0.0, x0, 0.0), [1e-3] * steps)
    assert res.status == "complete", res.error
    keys = sorted(res.diagnostics[0])
    save("config1_64", x0=x0, steps=steps, seed=2024, x_final=model.vector(res.final), r_final=res.final.r,
         t_final=res.final.t, diag_keys=np.array(keys), diagnostics=np.array([[d[k] for k in keys]
                                                                                for d in res.diagnostics]),
         iterations=np.array(model.backend.total_iterations))


def adaptive() -> None:
    """integrate_adaptive with the tensor backend: I control (the reference
    test's controls) and PI control on a rectangle, seeded periodic forcing."""
    from solver.adaptivity import IController, PIController, integrate_adaptive
    cases = {"i_sdirk3": (12, 10, 1.3, 0.8, "sdirk3", dict(atol=1e-12, rtol=1e-8, min_step=1e-7, max_step=.002),
                          False, 0.002, 0.002),
             "pi_sdirk3_mrsav": (32, 16, 2.0, 1.0, "sdirk3_mrsav", dict(rtol=1e-5, atol=1e-8), True, 0.01, 1e-3)}
    out = {}
    for tag, (nx, ny, lx, ly, scheme, ctl, pi, T, dt0) in cases.items():
        g = MACGrid(nx, ny, lx, ly)
        base = np.random.default_rng(nx * ny).normal(size=g.size)
        model = MACNavierStokes(g, 0.1 if nx == 12 else 5e-3)
        model.backend = TensorStokes(model.ops, tolerance=1e-9, krylov_tolerance=1e-12)
        model.force = lambda t, base=base: np.cos(2.0 * t) * base
        x0 = 0.2 * fields.packed_curl_velocity(nx, ny, lx, ly, 3, 5)
        controller = (PIController if pi else IController)(**ctl)
        res = integrate_adaptive(model, make_scheme(scheme), model.state(0.0, x0, 0.1 if "mrsav" in scheme else 0.0),
                                 T, dt0, controller=controller)
        assert res.status == "complete", res.error
        out.update({f"{tag}_shape": [nx, ny, lx, ly], f"{tag}_base": base, f"{tag}_x0": x0,
                    f"{tag}_accepted": np.array([a["accepted"] for a in res.attempts]),
                    f"{tag}_steps": np.array([a["step"] for a in res.attempts]),
                    f"{tag}_errors": np.array([a["error"] for a in res.attempts]),
                    f"{tag}_x_final": model.vector(res.final), f"{tag}_r_final": res.final.r,
                    f"{tag}_t_final": res.final.t, f"{tag}_nu": model.nu})
    save("adaptive", **out)


def channel() -> None:
    """Channel MAC (periodic x): FFTStokes solves on the reference tests'
    shapes and shifts, convection of a random field, and a short
    integration of two schemes on the FFT-backed ChannelModel."""
    from solver.channel import ChannelGrid, ChannelModel
    from solver.channel.kernels import convection as ch_conv
    out = {}
    for nx, ny in ((7, 5), (8, 6), (17, 9)):
        grid = ChannelGrid(nx, ny, 2.3, .8)
        model = ChannelModel(grid, .1, backend="fft")
        loads = np.random.default_rng(54).normal(size=(grid.size, 2))
        for k, (mass, alpha) in enumerate(((1., 0.), (1., .013), (0., .2))):
            sol = model.solve(loads, mass=mass, viscosity=alpha)
            tag = f"solve_{nx}x{ny}_{k}"
            out.update({f"{tag}_loads": loads, f"{tag}_shift": [mass, alpha], f"{tag}_vel": sol.velocity,
                        f"{tag}_pres": sol.pressure, f"{tag}_res": sol.residual, f"{tag}_div": sol.divergence_inf})
    grid = ChannelGrid(9, 7, 2., .8)
    model = ChannelModel(grid, .1)
    w = np.random.default_rng(43).normal(size=grid.size)
    u, v = grid.unpack(w)
    out.update({"conv_w": w, "conv_n": grid.pack(*ch_conv(u, v, grid.hx, grid.hy)),
                "conv_K": model.apply_K(w), "conv_D": model.apply_D(w),
                "conv_G": model.apply_G(np.random.default_rng(44).normal(size=grid.np)),
                "conv_p": np.random.default_rng(44).normal(size=grid.np)})
    grid = ChannelGrid(12, 9, 2 * np.pi, 1.)
    x, y = grid.coordinates("vertex")
    psi = (np.sin(2 * np.pi * x / grid.lx) + .3 * np.cos(4 * np.pi * x / grid.lx)) * np.sin(np.pi * y / grid.ly) ** 2
    psi[[0, -1]] = 0.
    x0 = .5 * grid.curl(psi)
    out["run_x0"] = x0
    for name in ("sdirk2_mrsav", "sdirk3"):
        model = ChannelModel(grid, .1, backend="fft")
        res = integrate(model, make_scheme(name, 1000.), model.state(0., x0, 1.0 if "mrsav" in name else 0.),
                        [.01, .02, .01])
        assert res.status == "complete", res.error
        out.update({f"run_{name}_x": model.vector(res.final), f"run_{name}_r": res.final.r,
                    f"run_{name}_p": np.array([s.pressure for s in res.final_stages]),
                    f"run_{name}_diag": np.array([res.diagnostics[-1][k] for k in sorted(res.diagnostics[-1])]),
                    f"run_{name}_diag_keys": np.array(sorted(res.diagnostics[-1]))})
    save("channel", **out)


if __name__ == "__main__":
    channel()
    adaptive()
    operators()
    stokes()
    scalar()
    schemes()
    config1()
    (HERE / "SOURCE.json").write_text(json.dumps({
        "generator": "tests/golden/make_golden.py",
        "reference": "HaifengWang1031/MAC-mr-SAV-RK (solver/ imported unchanged, numba.njit -> identity)",
        "numpy": np.__version__, "scipy": __import__("scipy").__version__}, indent=1) + "\n")
