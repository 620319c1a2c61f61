"""FP32 row transforms (macsav_transform32): the shared-memory FFT and the
tcgen05 transform-matrix products against scipy.fft (norm="ortho", the
transforms the reference applies, solver/mac/tensor_stokes.py:58-82), and the
per-size autotuner.

Bars (relative L2 against scipy in FP64 on the same FP32 inputs): FFT and
the 6-product split (TC6) 5e-6, the FP32 class; the 3-product split (TC3)
1e-4 (about 16 mantissa bits).
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from helpers import load_package

pytestmark = pytest.mark.gpu

FFT, TC3, TC6, AUTO = 0, 1, 2, 3
BARS = {FFT: 5e-6, TC3: 1e-4, TC6: 5e-6}
NAMES = {0: "dct2", 1: "dst2", 2: "dst1"}


@pytest.fixture(scope="module")
def env():
    import torch
    from importlib import import_module
    pkg = load_package()
    stokes = import_module(pkg.__name__ + ".stokes")
    lib = import_module(pkg.__name__ + "._lib")
    plan = stokes.Plan(pkg.MACGrid(8, 8))
    return pkg, stokes, lib, torch, plan


def _run(env, kind, inverse, a, method):
    pkg, stokes, lib, torch, plan = env
    x = torch.as_tensor(a, dtype=torch.float32, device="cuda").contiguous()
    out = torch.empty_like(x)
    rows, n = a.shape
    code = plan.lib.macsav_transform32(plan.handle, kind, inverse, rows, n, method, stokes.dptr(x), stokes.dptr(out),
                                       stokes.stream_handle())
    return code, out.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("kind", [0, 1, 2])
@pytest.mark.parametrize("n", [2, 7, 16, 63, 64, 96, 127, 255, 256, 300, 511, 512])
def test_transform32_methods_match_scipy(env, kind, n):
    pkg, stokes, lib, torch, plan = env
    rows = 130  # one full 128-row tile and a ragged one
    a = np.random.default_rng(n * 3 + kind).normal(size=(rows, n)).astype(np.float32).astype(np.float64)
    for inverse in (0, 1):
        ref = O.trig_transform(a, NAMES[kind], 1, bool(inverse))
        for method in (FFT, TC3, TC6):
            code, got = _run(env, kind, inverse, a, method)
            assert code == lib.OK, plan.lib.macsav_plan_error(plan.handle)
            err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
            assert err <= BARS[method], (kind, n, inverse, method, err)


def test_autotuner_choice_and_auto_method(env):
    pkg, stokes, lib, torch, plan = env
    for kind, n, rows in ((0, 64, 4096), (2, 511, 1024), (1, 256, 2048)):
        m, t_fft, t_tc = C.c_int(), C.c_double(), C.c_double()
        code = plan.lib.macsav_transform32_autotune(plan.handle, kind, 0, rows, n, C.byref(m), C.byref(t_fft),
                                                    C.byref(t_tc), stokes.stream_handle())
        assert code == lib.OK
        assert m.value in (FFT, TC6) and t_fft.value > 0 and t_tc.value > 0
        assert (m.value == TC6) == (t_tc.value < t_fft.value)
        print(f"kind {kind} n {n} rows {rows}: FFT {t_fft.value * 1e3:.1f} us, TC6 {t_tc.value * 1e3:.1f} us, "
              f"chosen {'TC6' if m.value == TC6 else 'FFT'}")
        a = np.random.default_rng(1).normal(size=(rows, n)).astype(np.float32).astype(np.float64)
        code, auto = _run(env, kind, 0, a, AUTO)
        assert code == lib.OK
        code, chosen = _run(env, kind, 0, a, m.value)
        np.testing.assert_array_equal(auto, chosen)


def test_tensor_forms_reject_long_lines_fft_takes_them(env):
    pkg, stokes, lib, torch, plan = env
    a = np.random.default_rng(2).normal(size=(4, 1024))
    code, _ = _run(env, 0, 0, a, TC6)
    assert code == lib.ERR_UNSUPPORTED
    code, got = _run(env, 0, 0, a, FFT)
    assert code == lib.OK
    ref = O.trig_transform(a.astype(np.float32).astype(np.float64), "dct2", 1, False)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < BARS[FFT]
    m, t_fft, t_tc = C.c_int(), C.c_double(), C.c_double()
    assert plan.lib.macsav_transform32_autotune(plan.handle, 0, 0, 4, 1024, C.byref(m), C.byref(t_fft),
                                                C.byref(t_tc), stokes.stream_handle()) == lib.OK
    assert m.value == FFT and t_tc.value == -1.0
