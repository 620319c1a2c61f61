"""FP64 and FP32-bulk parity against the oracle at the workloads' full sizes.

The small-grid parity tests pin the CUDA path to the reference's own fixtures;
these send the compile-time-length transform passes the full-size workloads
use (k_column_p2 / k_row_*_p2 at 512, 1024 and 2048 points) through the
oracle (a NumPy/SciPy restatement of solver/mac/tensor_stokes.py:245-364 and
solver/schemes/sdirk3_mrsav.py:18-65, itself pinned to fixtures the reference
produced):

* one sdirk3_mrsav step of the 512^2 precision case (nu=1e-3, dt=2.5e-4,
  stream-function modes k,l <= 16);
* one two-column Stokes solve at 1024^2 with the learned-preconditioner
  case's stage shift (nu=1e-4, dt=1e-4: mass 1, viscosity nu dt / 4), Krylov
  tolerance 1e-12;
* one two-column Stokes solve on the 2048 x 1024 rectangle [0,2] x [0,1] of
  the adaptive case (nu=5e-5, dt=1e-4).

Bars: FP64 within 1e-11 relative L2 in u, v and p of the oracle with identical
CG iteration counts; FP32 bulk within 1e-6 (the precision budget of the FP32
form; it lands near 1e-13).  The right-hand sides are the two columns a stage
solves: the seeded curl field (discretely divergence-free) and its
convection.

The pressure of a divergence-free right-hand side is only the wall
commutator's response, about 1e-10 of the velocity here, and it is fixed by
the data only to rounding of the velocity (eps |f| / h): its own relative
difference between two correct FP64 codes is 1e-7..1e-6.  For such a pressure
the bar applies to what it does in the momentum equation, the gradient:
|D^T (p - p_ref)| <= bar |f|.  Pressures that carry the right-hand side (the
convection column) meet the plain relative bar.  A stage multiplier is
pi_V / dt - coupling pi_W; with the SAV scalar near 1 the coupling is small
and pi is mostly the divergence-free column's response, so it takes the
gradient form (dt |D^T (pi - pi_ref)| <= bar |U|) when dt |D^T pi| is below
1e-3 |U| (here about 2e-6 |U|: the multiplier carries a few millionths of the
momentum balance and its own relative difference, 2e-10, is rounding of the
divergence-free column), and the plain relative bar otherwise.
"""
import numpy as np
import pytest

import oracle as O
from helpers import load_package

pytestmark = pytest.mark.gpu

SEED = 20261203


@pytest.fixture(scope="module")
def pkg():
    return load_package()


class _CountingOracle(O.TensorStokesOracle):
    """The oracle backend, keeping the CG iteration counts of every solve."""

    def __init__(self, *a, **k):
        super().__init__(*a, **k)
        self.history = []

    def solve(self, rhs, *, mass, viscosity):
        out = super().solve(rhs, mass=mass, viscosity=viscosity)
        self.history.append(tuple(self.last_iterations))
        return out


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _parts(g, x):
    n_u = g.n_u if hasattr(g, "n_u") else g.nu  # the oracle's grid names it n_u
    return x[:n_u], x[n_u:]


def _stage_rhs(og, pkg, nx, ny, lx, ly, modes, dt):
    x0 = pkg.fields.packed_curl_velocity(nx, ny, lx, ly, modes, SEED)
    return np.column_stack([x0, dt * O.nonlinear(og, x0)])


def _grad_rel(og, p, p_ref, f):
    """|D^T (p - p_ref)| / |f|: the pressure difference as a momentum defect."""
    dp = (np.asarray(p) - np.asarray(p_ref)).ravel()
    return float(np.linalg.norm(O.apply_Dt(og, dp)) / np.linalg.norm(f))


def _check_solve(pkg, shape, nu, dt, modes):
    nx, ny, lx, ly = shape
    og = O.Grid(nx, ny, lx, ly)
    g = pkg.MACGrid(nx, ny, lx, ly)
    rhs = _stage_rhs(og, pkg, nx, ny, lx, ly, modes, dt)
    mass, visc = 1.0, nu * dt / 4
    ref_solver = O.TensorStokesOracle(og, 1e-9, 1e-12)
    ref = ref_solver.solve(rhs, mass=mass, viscosity=visc)
    from importlib import import_module
    stokes = import_module(pkg.__name__ + ".stokes")
    for precision, bar in (("fp64", 1e-11), ("fp32", 1e-6)):
        solver = stokes.TensorStokes(g, tolerance=1e-9, krylov_tolerance=1e-12, precision=precision)
        got = solver.solve(rhs, mass=mass, viscosity=visc)
        for c in range(2):
            gu, gv = _parts(g, got.velocity[:, c])
            ru, rv = _parts(g, ref.velocity[:, c])
            gp, rp = got.pressure[:, :, c], ref.pressure[:, :, c]
            # column 0 is divergence-free: its pressure is checked through its gradient
            perr = _rel(gp, rp) if c == 1 else _grad_rel(og, gp, rp, rhs[:, c])
            errs = (_rel(gu, ru), _rel(gv, rv), perr, _grad_rel(og, gp, rp, rhs[:, c]))
            assert max(errs) <= bar, (precision, c, errs)
        if precision == "fp64":
            assert solver.last_iterations == ref_solver.last_iterations
        assert got.residual <= 1e-9 and got.divergence_inf <= 1e-9 * (1 + np.abs(got.velocity).max())


def test_fp64_solve_1024_learned_case_shift_matches_oracle(pkg):
    _check_solve(pkg, (1024, 1024, 1.0, 1.0), 1e-4, 1e-4, 32)


def test_fp64_solve_2048x1024_matches_oracle(pkg):
    _check_solve(pkg, (2048, 1024, 2.0, 1.0), 5e-5, 1e-4, 64)


def test_sdirk3_mrsav_step_512_matches_oracle(pkg):
    """One graph-captured fused step of the 512^2 precision case in FP64 and
    in FP32 bulk against the oracle's step (same initial field, r0 = 1)."""
    nx = ny = 512
    nu, dt = 1e-3, 2.5e-4
    og = O.Grid(nx, ny)
    x0 = pkg.fields.packed_curl_velocity(nx, ny, 1.0, 1.0, 16, SEED)
    backend = _CountingOracle(og, 1e-9, 1e-12)
    om = O.OracleModel(og, nu, backend=backend)
    ref = O.make_scheme("sdirk3_mrsav").step(om, om.state(0.0, x0, 1.0), dt)
    rx = om.vector(ref.state)
    ru, rv = _parts(og, rx)
    g = pkg.MACGrid(nx, ny)
    for precision, bar in (("fp64", 1e-11), ("fp32", 1e-6)):
        model = pkg.MACNavierStokes(g, nu, precision=precision, use_graph=True)
        trial = pkg.make_scheme("sdirk3_mrsav").step(model, model.state(0.0, x0, 1.0), dt)
        x = model.vector(trial.state)
        gu, gv = _parts(g, x)
        assert max(_rel(gu, ru), _rel(gv, rv)) <= bar, precision
        assert abs(trial.state.r - ref.state.r) <= (1e-12 if precision == "fp64" else 1e-9)
        assert len(trial.stages) == len(ref.stages) == 4
        for k, (sg, sr) in enumerate(zip(trial.stages, ref.stages)):
            gp, rp = np.asarray(sg.pressure), np.asarray(sr.pressure)
            # dt |D^T pi| against |U|: how much momentum the stage multiplier carries
            weight = dt * np.linalg.norm(O.apply_Dt(og, rp.ravel())) / np.linalg.norm(x0)
            perr = _rel(gp, rp) if weight > 1e-3 else dt * _grad_rel(og, gp, rp, x0)
            assert perr <= bar, (precision, k, perr, weight)
            assert abs(sg.r - sr.r) <= (1e-12 if precision == "fp64" else 1e-9)
            if precision == "fp64":
                assert tuple(sg.iterations) == backend.history[k], (k, sg.iterations, backend.history[k])
        if precision == "fp64":
            emb = trial.embedded_velocity.cpu().numpy()
            assert _rel(emb, ref.embedded_velocity) <= 1e-11
        del model
