"""Adaptive stepping against the reference's own adaptive runs (golden fixture:
I control on sdirk3 and PI control on sdirk3_mrsav, with a time-dependent
body force).

* CPU: the restatement of the reference's driver (oracle/adaptive_oracle.py,
  solver/adaptivity/controller.py:126-398) on the oracle model pins that
  restatement to the reference;
* GPU: the same driver on the GPU model and the fused schemes, i.e. the
  package dropped in behind the reference's driver;
* GPU: the package's device-resident loop ``run_adaptive``, given the
  reference's controller objects.

Bars: the accept/reject sequence equal, steps within 2e-8 (the embedded
error at rtol 1e-8 carries about 1e-8 relative rounding noise into each
proposed step; the reference bounds its Tensor-vs-Direct steps at 2e-8), the
final time exact and the final state within 2e-11.
"""
import numpy as np
import pytest

import oracle as O
import oracle.adaptive_oracle as A
from helpers import golden, load_package

CASES = {"i_sdirk3": ("sdirk3", False, dict(atol=1e-12, rtol=1e-8, min_step=1e-7, max_step=.002), 0.002, 0.002),
         "pi_sdirk3_mrsav": ("sdirk3_mrsav", True, dict(rtol=1e-5, atol=1e-8), 0.01, 1e-3)}


def _check(attempts, final, d, tag, vector):
    np.testing.assert_array_equal([a["accepted"] for a in attempts], d[f"{tag}_accepted"])
    np.testing.assert_allclose([a["step"] for a in attempts], d[f"{tag}_steps"], rtol=2e-8, atol=1e-11)
    assert final.t == float(d[f"{tag}_t_final"])
    np.testing.assert_allclose(vector(final), d[f"{tag}_x_final"], rtol=2e-11, atol=2e-11)


def _case(tag):
    d = golden("adaptive")
    scheme, pi, ctl, T, dt0 = CASES[tag]
    nx, ny, lx, ly = d[f"{tag}_shape"]
    base = d[f"{tag}_base"]
    r0 = 0.1 if "mrsav" in scheme else 0.0
    controller = (A.PIController if pi else A.IController)(**ctl)
    return d, scheme, controller, T, dt0, (int(nx), int(ny), float(lx), float(ly)), base, r0


@pytest.mark.parametrize("tag", list(CASES))
def test_reference_driver_with_oracle_model_matches_reference(tag):
    d, scheme, controller, T, dt0, shape, base, r0 = _case(tag)
    g = O.Grid(*shape)
    model = O.OracleModel(g, float(d[f"{tag}_nu"]), force=lambda t: np.cos(2.0 * t) * base,
                          backend=O.TensorStokesOracle(g, 1e-9, 1e-12))
    res = A.integrate_adaptive(model, O.make_scheme(scheme), model.state(0.0, d[f"{tag}_x0"], r0), T, dt0,
                               controller=controller)
    assert res.status == "complete", res.error
    _check(res.attempts, res.final, d, tag, model.vector)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", list(CASES))
def test_gpu_model_behind_reference_driver_matches_reference(tag):
    pkg = load_package()
    d, scheme, controller, T, dt0, shape, base, r0 = _case(tag)
    model = pkg.MACNavierStokes(pkg.MACGrid(*shape), float(d[f"{tag}_nu"]),
                                force=lambda t: np.cos(2.0 * t) * base, use_graph=True)
    res = A.integrate_adaptive(model, pkg.make_scheme(scheme), model.state(0.0, d[f"{tag}_x0"], r0), T, dt0,
                               controller=controller)
    assert res.status == "complete", res.error
    _check(res.attempts, res.final, d, tag, model.vector)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", list(CASES))
def test_device_loop_matches_reference(tag):
    pkg = load_package()
    d, scheme, controller, T, dt0, shape, base, r0 = _case(tag)
    model = pkg.MACNavierStokes(pkg.MACGrid(*shape), float(d[f"{tag}_nu"]),
                                force=lambda t: np.cos(2.0 * t) * base, use_graph=True)
    run = pkg.run_adaptive(model, pkg.make_scheme(scheme), model.state(0.0, d[f"{tag}_x0"], r0), T, dt0,
                           controller)
    assert run.status == "complete", run.error
    assert run.attempted_steps == len(d[f"{tag}_accepted"])
    assert run.accepted_steps == int(np.sum(d[f"{tag}_accepted"]))
    _check(run.attempts, run.final, d, tag, model.vector)


def test_step_control_reads_reference_controllers_and_validates():
    """StepControl.of takes the reference controllers' parameters; its
    factors follow the controller formulas (controller.py:14-70)."""
    pkg = load_package()
    from importlib import import_module
    D = import_module(pkg.__name__ + ".drive")
    pi = D.StepControl.of(A.PIController(rtol=1e-5, atol=1e-8))
    ref = A.PIController(rtol=1e-5, atol=1e-8)
    for err, prev in ((0.3, None), (0.3, 0.7), (1e-16, 2.0), (0.99, 1e-20)):
        assert pi.grow(err, prev) == ref.accepted_factor(err, prev)
    el = D.StepControl.of(A.IController(atol=1e-12, rtol=1e-8))
    for err in (0.0, 0.5, 3.0, float("inf")):
        assert el.grow(err, 0.4) == A.IController(atol=1e-12, rtol=1e-8).accepted_factor(err, 0.4)
        assert el.shrink(err) == min(A.IController(atol=1e-12, rtol=1e-8).accepted_factor(err, None), 0.8)
    assert el.error(4.0, 1.0, 9.0) == 2.0 / (1e-12 + 1e-8 * 3.0)
    assert el.error(float("nan"), 1.0, 1.0) == float("inf")
    for bad in (dict(atol=0.0, rtol=0.0), dict(safety=1.5), dict(min_step=0.0), dict(order=1), dict(pi=(0.2, 0.4))):
        with pytest.raises(ValueError):
            D.StepControl(**bad)


def test_step_control_factors_equal_the_controllers_over_a_seeded_sweep():
    """Over seeded errors from 1e-20 to 1e6 (and exact zeros), the package's
    step factors equal the reference controllers' bit for bit: accepted
    (I and PI, with and without a previous error) and rejected (the I factor
    capped at 0.8, controller.py:276 in the driver)."""
    pkg = load_package()
    from importlib import import_module
    D = import_module(pkg.__name__ + ".drive")
    rng = np.random.default_rng(11)
    errs = np.concatenate([[0.0, 1.0, 1e-14, 1e-15], 10.0 ** rng.uniform(-20, 6, 2000)])
    prevs = np.concatenate([[0.0, 1.0, 1e-15, 1e-14], 10.0 ** rng.uniform(-20, 6, 2000)])
    for ref in (A.IController(atol=1e-10, rtol=1e-6, max_step=0.01), A.PIController(rtol=1e-5, atol=1e-8),
                A.PIController(rtol=1e-4, atol=0.0, proportional=0.6, integral=0.2, safety=0.8, min_factor=0.1,
                               max_factor=5.0, estimator_order=2)):
        ctl = D.StepControl.of(ref)
        for e, p in zip(errs, prevs):
            e, p = float(e), float(p)
            assert ctl.grow(e, None) == ref.accepted_factor(e, None)
            assert ctl.grow(e, p) == ref.accepted_factor(e, p)
            assert ctl.shrink(e) == min(A.IController.accepted_factor(ref, e, None), 0.8)
