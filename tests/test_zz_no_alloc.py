"""macsav_inner_max_static: the plan-free reduction with static scratch.

Collected last on purpose, so that it also runs after every other GPU test in
the same process; it must pass alone in a fresh process too.  Each check makes
two calls in a row and compares them with the plan-based entry points
macsav_inner / macsav_max_abs (dot product to rounding, maximum exactly).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_package

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from importlib import import_module
    pkg = load_package()
    stokes = import_module(pkg.__name__ + ".stokes")
    lib = import_module(pkg.__name__ + "._lib")
    return pkg, stokes, lib, torch


def _static(env, a, b, n, weight):
    pkg, stokes, lib, torch = env
    out = (C.c_double * 2)()
    code = lib.load().macsav_inner_max_static(stokes.dptr(a), stokes.dptr(b) if b is not None else None, n,
                                              float(weight), out, stokes.stream_handle())
    return code, out[0], out[1]


def _planned(env, plan, a, b, n):
    pkg, stokes, lib, torch = env
    inner, mx = C.c_double(), C.c_double()
    plan.check(plan.lib.macsav_inner(plan.handle, stokes.dptr(a), stokes.dptr(b), n, C.byref(inner),
                                     stokes.stream_handle()))
    plan.check(plan.lib.macsav_max_abs(plan.handle, stokes.dptr(a), n, C.byref(mx), stokes.stream_handle()))
    return inner.value, mx.value


@pytest.mark.parametrize("nx,ny", [(512, 512), (96, 64), (2048, 1024)])
def test_matches_plan_reduction_twice(env, nx, ny):
    pkg, stokes, lib, torch = env
    grid = pkg.MACGrid(nx, ny, nx / ny, 1.0)
    plan = stokes.Plan(grid)
    gen = torch.Generator(device="cuda").manual_seed(nx * 7 + ny)
    x = torch.randn(grid.size, dtype=torch.float64, device="cuda", generator=gen)
    y = torch.randn(grid.size, dtype=torch.float64, device="cuda", generator=gen)
    w = grid.hx * grid.hy
    inner, mx = _planned(env, plan, x, y, grid.size)
    for _ in range(2):
        code, s_inner, s_max = _static(env, x, y, grid.size, w)
        assert code == lib.OK
        assert s_inner == pytest.approx(inner, rel=1e-12, abs=1e-14 * w * grid.size)
        assert s_max == mx


def test_sum_form_ragged_and_empty(env):
    pkg, stokes, lib, torch = env
    plan = stokes.Plan(pkg.MACGrid(16, 12))
    for n in (0, 1, 4095, 4097, 100003):
        a = torch.linspace(-1.0, 2.0, max(n, 1), dtype=torch.float64, device="cuda")
        for _ in range(2):
            code, s_sum, s_max = _static(env, a, None, n, 1.0)
            assert code == lib.OK
            ref_sum = float(a[:n].sum()) if n else 0.0
            assert s_sum == pytest.approx(ref_sum, rel=1e-12, abs=1e-12)
            if n:
                _, p_max = _planned(env, plan, a, a, n)
                assert s_max == p_max
            else:
                assert s_max == 0.0


def test_nan_propagates_like_max_abs(env):
    pkg, stokes, lib, torch = env
    plan = stokes.Plan(pkg.MACGrid(16, 12))
    a = torch.randn(50000, dtype=torch.float64, device="cuda")
    a[31337] = float("nan")
    _, p_max = _planned(env, plan, a, a, a.numel())
    for _ in range(2):
        code, _, s_max = _static(env, a, None, a.numel(), 1.0)
        assert code == lib.OK
        assert np.isnan(s_max) and np.isnan(p_max)


def test_rejects_sizes_beyond_the_static_limit(env):
    pkg, stokes, lib, torch = env
    a = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = (C.c_double * 2)(-1.0, -1.0)
    handle = lib.load()
    # rejected on the host before any device work, so the short buffer is never read
    code = handle.macsav_inner_max_static(stokes.dptr(a), None, lib.STATIC_REDUCE_MAX_N + 1, 1.0, out,
                                          stokes.stream_handle())
    assert code == lib.ERR_UNSUPPORTED and out[0] == -1.0
    assert handle.macsav_inner_max_static(stokes.dptr(a), None, -1, 1.0, out, stokes.stream_handle()) == lib.ERR_VALUE
    assert handle.macsav_inner_max_static(None, None, 8, 1.0, out, stokes.stream_handle()) == lib.ERR_VALUE
