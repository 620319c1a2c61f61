"""The C-ABI library builds for sm_103a and exports every declared symbol
(no GPU needed: nothing here launches a kernel)."""
import ctypes

from helpers import load_package


def _lib_module():
    import __graft_entry__
    __graft_entry__.build()
    pkg = load_package()
    from importlib import import_module
    return import_module(pkg.__name__ + "._lib")


def test_library_exports_every_header_symbol():
    lib = _lib_module()
    names = lib.header_symbols()
    assert "macsav_stokes_solve" in names and "macsav_plan_create" in names
    so = ctypes.CDLL(str(lib.LIB_PATH))
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing
    # every declared symbol also has a ctypes signature in the binding
    assert set(names) <= set(lib._SIGNATURES), set(names) - set(lib._SIGNATURES)


def test_plan_create_rejects_bad_arguments_without_gpu():
    lib = _lib_module()
    so = lib.load()
    h = ctypes.c_void_p()
    assert so.macsav_plan_create(ctypes.byref(h), 2, 5, 1.0, 1.0, 0, 1e-9, 1e-12, 100, 2) == lib.ERR_VALUE
    assert b"nx,ny >= 3" in so.macsav_plan_error(None)
    assert so.macsav_plan_create(ctypes.byref(h), 8, 8, 1.0, 1.0, 0, -1.0, 1e-12, 100, 2) == lib.ERR_VALUE
    assert b"Invalid solver controls" in so.macsav_plan_error(None)
    assert not h.value


def test_host_mapped_rejects_bad_arguments_and_pageable_memory():
    import numpy as np
    lib = _lib_module()
    so = lib.load()
    a = np.zeros(1024)
    ok = ctypes.c_int(7)
    assert so.macsav_host_mapped(a.ctypes.data, a.nbytes, None) == lib.ERR_VALUE
    assert so.macsav_host_mapped(a.ctypes.data, -1, ctypes.byref(ok)) == lib.ERR_VALUE
    assert so.macsav_host_mapped(None, 8, ctypes.byref(ok)) == lib.OK and ok.value == 0
    # ordinary (pageable) host memory is never reported as mapped pinned memory
    ok.value = 7
    assert so.macsav_host_mapped(a.ctypes.data, a.nbytes, ctypes.byref(ok)) == lib.OK and ok.value == 0


def test_tuning_controls_reject_a_missing_plan_without_gpu():
    """The launch-shape controls and the pass timer validate their plan
    before touching the device."""
    lib = _lib_module()
    so = lib.load()
    ms, nbytes = ctypes.c_double(), ctypes.c_double()
    chosen = (ctypes.c_int * 6)()
    assert so.macsav_plan_set_launch_shape(None, 0) == lib.ERR_VALUE
    assert so.macsav_plan_autotune_launch_shapes(None, 10, chosen, None) == lib.ERR_VALUE
    assert so.macsav_time_pass(None, 0, 3, ctypes.byref(ms), ctypes.byref(nbytes), None) == lib.ERR_VALUE
