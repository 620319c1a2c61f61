"""Adaptive driver (the reference's solver/adaptivity/controller.py) against the
reference's own adaptive runs (golden fixture).  The CPU test drives the
host-side driver with the oracle model; the GPU test drives it with the GPU
model and the fused device scheme."""
import numpy as np
import pytest

import oracle as O
from helpers import golden, load_package

CASES = {"i_sdirk3": ("sdirk3", False, dict(atol=1e-12, rtol=1e-8, min_step=1e-7, max_step=.002), 0.002, 0.002),
         "pi_sdirk3_mrsav": ("sdirk3_mrsav", True, dict(rtol=1e-5, atol=1e-8), 0.01, 1e-3)}


def _check(res, d, tag, vector):
    assert res.status == "complete", res.error
    np.testing.assert_array_equal([a["accepted"] for a in res.attempts], d[f"{tag}_accepted"])
    # the embedded error at rtol 1e-8 carries ~1e-8 relative rounding noise into
    # each proposed step (the reference bounds Tensor-vs-Direct steps at 2e-8)
    np.testing.assert_allclose([a["step"] for a in res.attempts], d[f"{tag}_steps"], rtol=2e-8, atol=1e-11)
    assert res.final.t == float(d[f"{tag}_t_final"])
    np.testing.assert_allclose(vector(res.final), d[f"{tag}_x_final"], rtol=2e-11, atol=2e-11)


@pytest.mark.parametrize("tag", list(CASES))
def test_adaptive_driver_with_oracle_model_matches_reference(tag):
    pkg = load_package()
    from importlib import import_module
    A = import_module(pkg.__name__ + ".adaptivity")
    d = golden("adaptive")
    scheme, pi, ctl, T, dt0 = CASES[tag]
    nx, ny, lx, ly = d[f"{tag}_shape"]
    g = O.Grid(int(nx), int(ny), float(lx), float(ly))
    base = d[f"{tag}_base"]
    model = O.OracleModel(g, float(d[f"{tag}_nu"]), force=lambda t: np.cos(2.0 * t) * base,
                          backend=O.TensorStokesOracle(g, 1e-9, 1e-12))
    r0 = 0.1 if "mrsav" in scheme else 0.0
    res = A.integrate_adaptive(model, O.make_scheme(scheme), model.state(0.0, d[f"{tag}_x0"], r0), T, dt0,
                               controller=(A.PIController if pi else A.IController)(**ctl))
    _check(res, d, tag, model.vector)


@pytest.mark.gpu
@pytest.mark.parametrize("tag", list(CASES))
def test_adaptive_driver_on_gpu_matches_reference(tag):
    pkg = load_package()
    from importlib import import_module
    A = import_module(pkg.__name__ + ".adaptivity")
    d = golden("adaptive")
    scheme, pi, ctl, T, dt0 = CASES[tag]
    nx, ny, lx, ly = d[f"{tag}_shape"]
    g = pkg.MACGrid(int(nx), int(ny), float(lx), float(ly))
    base = d[f"{tag}_base"]
    model = pkg.MACNavierStokes(g, float(d[f"{tag}_nu"]), force=lambda t: np.cos(2.0 * t) * base, use_graph=True)
    r0 = 0.1 if "mrsav" in scheme else 0.0
    res = A.integrate_adaptive(model, pkg.make_scheme(scheme), model.state(0.0, d[f"{tag}_x0"], r0), T, dt0,
                               controller=(A.PIController if pi else A.IController)(**ctl))
    _check(res, d, tag, model.vector)
