"""The adaptive attempt loop on the device (``run_adaptive_device``,
``macsav_integrate_adaptive``: attempts, accept/reject, retries and step
proposals inside one CUDA graph launch) against

* the restatement of the reference's driver (oracle/adaptive_oracle.py,
  solver/adaptivity/controller.py:126-398, pinned to the reference's own
  adaptive runs in tests/test_adaptivity.py) on the oracle model;
* the package's host-driven loop ``run_adaptive`` on the same GPU model.

Cases are autonomous (no body force, as the device loop requires): a seeded
curl field on 48 x 32 cells of [0, 1.5] x [0, 1], a first step far too large
(so the loop rejects and retries on the device), PI control on
sdirk3_mrsav and I control on sdirk2_mrsav.

Bars, against both: the accept/reject sequence equal; steps within 2e-8
(the embedded error is a difference of two close velocities, so the last-bit
differences of the step -- the device forms the step coefficients as
c0 + c1 dt -- reach each step factor as relative noise of 1e-10..1e-9, as in
test_adaptivity); final time exact; final state within 2e-11.
"""
import numpy as np
import pytest

import oracle as O
import oracle.adaptive_oracle as A
from helpers import load_package

pytestmark = pytest.mark.gpu

SHAPE = (48, 32, 1.5, 1.0)
CASES = {"pi_sdirk3_mrsav": ("sdirk3_mrsav", A.PIController(rtol=1e-5, atol=1e-8), 0.05, 0.05, 0.1),
         "i_sdirk2_mrsav": ("sdirk2_mrsav", A.IController(atol=1e-10, rtol=1e-6, max_step=0.01), 0.02, 0.02, 0.3)}
NU = 2e-3


@pytest.fixture(scope="module")
def pkg():
    return load_package()


def _x0(pkg):
    nx, ny, lx, ly = SHAPE
    return pkg.fields.packed_curl_velocity(nx, ny, lx, ly, 4, 11)


def _model(pkg, precision="fp64"):
    return pkg.MACNavierStokes(pkg.MACGrid(*SHAPE), NU, precision=precision, use_graph=True)


@pytest.mark.parametrize("tag", list(CASES))
def test_device_loop_matches_reference_driver_and_host_loop(pkg, tag):
    scheme_name, ctl, T, dt0, r0 = CASES[tag]
    x0 = _x0(pkg)
    og = O.Grid(*SHAPE)
    om = O.OracleModel(og, NU, backend=O.TensorStokesOracle(og, 1e-9, 1e-12))
    ref = A.integrate_adaptive(om, O.make_scheme(scheme_name), om.state(0.0, x0, r0), T, dt0, controller=ctl)
    assert ref.status == "complete", ref.error
    ref_acc = [a["accepted"] for a in ref.attempts]
    assert not all(ref_acc), "the case must exercise rejections"

    model = _model(pkg)
    scheme = pkg.make_scheme(scheme_name)
    dev = pkg.run_adaptive_device(model, scheme, model.state(0.0, x0, r0), T, dt0, ctl)
    assert dev.status == "complete", dev.error
    assert [a["accepted"] for a in dev.attempts] == ref_acc
    np.testing.assert_allclose([a["step"] for a in dev.attempts], [a["step"] for a in ref.attempts], rtol=2e-8)
    assert dev.final.t == ref.final.t
    np.testing.assert_allclose(model.vector(dev.final), om.vector(ref.final), rtol=2e-11, atol=2e-11)
    assert abs(dev.final.r - ref.final.r) <= 1e-11
    assert dev.accepted_steps == sum(ref_acc) and dev.attempted_steps == len(ref_acc)

    host = pkg.run_adaptive(model, scheme, model.state(0.0, x0, r0), T, dt0, ctl)
    assert [a["accepted"] for a in host.attempts] == ref_acc
    np.testing.assert_allclose([a["step"] for a in dev.attempts], [a["step"] for a in host.attempts], rtol=2e-8)
    np.testing.assert_allclose([a["error"] for a in dev.attempts], [a["error"] for a in host.attempts], rtol=1e-5)
    np.testing.assert_allclose(model.vector(dev.final), model.vector(host.final), rtol=2e-11, atol=2e-11)
    assert dev.times == pytest.approx(host.times, rel=2e-8)


def test_device_loop_failures_keep_the_accepted_state(pkg):
    x0 = _x0(pkg)
    model = _model(pkg)
    scheme = pkg.make_scheme("sdirk3_mrsav")
    # no rejection allowed: the first (too large) attempt ends the run
    run = pkg.run_adaptive_device(model, scheme, model.state(0.0, x0, 0.1), 0.05, 0.05,
                                  A.PIController(rtol=1e-5, atol=1e-8, max_rejections=0))
    assert run.status == "failed" and run.error == "error_exceeded"
    assert run.attempted_steps == 1 and run.accepted_steps == 0 and run.final.t == 0.0
    np.testing.assert_array_equal(model.vector(run.final), x0)
    # the accepted-step cap
    run = pkg.run_adaptive_device(model, scheme, model.state(0.0, x0, 0.1), 0.05, 1e-3,
                                  A.PIController(rtol=1e-5, atol=1e-8, max_steps=2))
    assert run.status == "failed" and run.error == "Maximum accepted steps exceeded"
    assert run.accepted_steps == 2 and 0.0 < run.final.t < 0.05


def test_device_loop_validates_like_the_host_loop(pkg):
    x0 = _x0(pkg)
    model = _model(pkg)
    scheme = pkg.make_scheme("sdirk3_mrsav")
    with pytest.raises(ValueError):
        pkg.run_adaptive_device(model, scheme, model.state(0.0, x0, 0.1), 0.05, 1e-12, A.PIController())
    with pytest.raises(ValueError):
        pkg.run_adaptive_device(model, scheme, model.state(0.0, x0, 0.1), -1.0, 1e-3)
    with pytest.raises(ValueError):
        pkg.run_adaptive_device(model, pkg.make_scheme("imex_euler_mrsav"), model.state(0.0, x0, 0.1), 0.05, 1e-3)
    forced = pkg.MACNavierStokes(pkg.MACGrid(*SHAPE), NU, force=lambda t: np.zeros(model.grid.size))
    with pytest.raises(ValueError):
        pkg.run_adaptive_device(forced, scheme, forced.state(0.0, x0, 0.1), 0.05, 1e-3)


def test_device_loop_fp32_bulk_follows_fp64(pkg):
    scheme_name, ctl, T, dt0, r0 = CASES["pi_sdirk3_mrsav"]
    x0 = _x0(pkg)
    runs = {}
    for precision in ("fp64", "fp32"):
        model = _model(pkg, precision)
        run = pkg.run_adaptive_device(model, pkg.make_scheme(scheme_name), model.state(0.0, x0, r0), T, dt0, ctl)
        assert run.status == "complete", run.error
        runs[precision] = (run, model.vector(run.final))
    a, b = runs["fp64"][0], runs["fp32"][0]
    assert [x["accepted"] for x in a.attempts] == [x["accepted"] for x in b.attempts]
    assert np.linalg.norm(runs["fp32"][1] - runs["fp64"][1]) <= 1e-9 * np.linalg.norm(runs["fp64"][1])
