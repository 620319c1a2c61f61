"""ctypes binding of ``libmacsav.so`` (the C ABI in include/macsav.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
Error codes are turned into the reference's exception types and messages.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import re

LIB_PATH = pathlib.Path(__file__).resolve().parent / "libmacsav.so"
HEADER = pathlib.Path(__file__).resolve().parent.parent / "include" / "macsav.h"

OK, ERR_VALUE, ERR_CUDA, ERR_CG, ERR_STOKES_GATE, ERR_STAGE_GATE, ERR_NEG_ENERGY, ERR_SCALAR, ERR_UNSUPPORTED = range(9)
FP64, FP32_MIXED = 0, 1
DCT2, DST2, DST1 = 0, 1, 2
MAX_COLUMNS = 4
STATIC_REDUCE_MAX_N = 16777216  # MACSAV_STATIC_REDUCE_MAX_N


class MacsavError(RuntimeError):
    """CUDA-side failure that has no counterpart in the reference."""


class StokesInfo(C.Structure):
    _fields_ = [("residual", C.c_double), ("divergence_inf", C.c_double), ("max_velocity", C.c_double),
                ("iterations", C.c_int * MAX_COLUMNS), ("refinements", C.c_int)]


class StepControl(C.Structure):
    """``macsav_step_control``."""
    _fields_ = [("atol", C.c_double), ("rtol", C.c_double), ("safety", C.c_double), ("min_factor", C.c_double),
                ("max_factor", C.c_double), ("min_step", C.c_double), ("max_step", C.c_double),
                ("error_floor", C.c_double), ("proportional", C.c_double), ("integral", C.c_double),
                ("order", C.c_int), ("max_rejections", C.c_int), ("max_steps", C.c_int), ("pad", C.c_int)]


class AdaptiveAttempt(C.Structure):
    """``macsav_adaptive_attempt``."""
    _fields_ = [("t", C.c_double), ("step", C.c_double), ("error", C.c_double), ("factor", C.c_double),
                ("accepted", C.c_int), ("reason", C.c_int), ("stage_status", C.c_int), ("pad", C.c_int)]


class AdaptiveResult(C.Structure):
    """``macsav_adaptive_result``."""
    _fields_ = [("t", C.c_double), ("r", C.c_double), ("next_step", C.c_double), ("status", C.c_int),
                ("reason", C.c_int), ("accepted_steps", C.c_int), ("attempted_steps", C.c_int)]


class StageRecord(C.Structure):
    """``macsav_stage_record``."""
    _fields_ = [("r", C.c_double), ("residual", C.c_double), ("scalar_residual", C.c_double),
                ("divergence_inf", C.c_double), ("continuity_residual", C.c_double),
                ("correction_predictor", C.c_double), ("frozen_factor", C.c_double),
                ("corrections", C.c_double * 2), ("stokes_residual", C.c_double),
                ("stokes_divergence", C.c_double), ("max_velocity", C.c_double), ("max_pressure", C.c_double),
                ("n_corrections", C.c_int), ("iterations", C.c_int * 2), ("cg_info", C.c_int), ("status", C.c_int)]


_P = C.c_void_p
_D = C.c_double
_I = C.c_int
_LL = C.c_longlong
_SIGNATURES = {
    "macsav_plan_create": (_I, [C.POINTER(_P), _I, _I, _D, _D, _I, _D, _D, _I, _I]),
    "macsav_plan_destroy": (None, [_P]),
    "macsav_plan_error": (C.c_char_p, [_P]),
    "macsav_plan_launches": (_LL, [_P]),
    "macsav_apply_K": (_I, [_P, _P, _P, _I, _P]),
    "macsav_apply_D": (_I, [_P, _P, _P, _I, _P]),
    "macsav_apply_Dt": (_I, [_P, _P, _P, _I, _P]),
    "macsav_convection": (_I, [_P, _P, _P, _I, _P]),
    "macsav_transform": (_I, [_P, _I, _I, _I, _I, _P, _P, _P]),
    "macsav_stokes_solve": (_I, [_P, _P, _I, _D, _D, _P, _P, C.POINTER(StokesInfo), _P]),
    "macsav_velocity_inverse": (_I, [_P, _P, _P, _I, _D, _D, _P]),
    "macsav_schur_precondition": (_I, [_P, _P, _P, _I, _D, _D, _P]),
    "macsav_combine": (_I, [_P, _I, C.POINTER(_D), C.POINTER(_P), _P, _LL, _P]),
    "macsav_inner": (_I, [_P, _P, _P, _LL, C.POINTER(_D), _P]),
    "macsav_max_abs": (_I, [_P, _P, _LL, C.POINTER(_D), _P]),
    "macsav_inner_max_static": (_I, [_P, _P, _LL, _D, C.POINTER(_D), _P]),
    "macsav_diagnostics": (_I, [_P, _P, _D, _D, _P, C.POINTER(_D), _P]),
    "macsav_step": (_I, [_P, _I, _D, _D, _D, _D, _P, _D, _P, _P, _P, _P, C.POINTER(StageRecord), C.POINTER(_D), _P]),
    "macsav_plan_set_graph": (_I, [_P, _I]),
    "macsav_unet_create": (_I, [C.POINTER(_P), _P]),
    "macsav_unet_destroy": (None, [_P]),
    "macsav_unet_error": (C.c_char_p, [_P]),
    "macsav_unet_num_params": (_LL, [_P]),
    "macsav_unet_set_params": (_I, [_P, _P]),
    "macsav_unet_get_params": (_I, [_P, _P]),
    "macsav_unet_forward": (_I, [_P, _P, _I, _I, _I, _P, _P]),
    "macsav_unet_set_tensor_cores": (_I, [_P, _I]),
    "macsav_unet_gradients": (_I, [_P, _P, _P, _I, _I, _I, C.POINTER(_D), _P, _P]),
    "macsav_unet_train_step": (_I, [_P, _P, _P, _I, _I, _I, C.c_float, C.POINTER(_D), _P]),
    "macsav_plan_set_preconditioner": (_I, [_P, _P, _I]),
    "macsav_plan_set_learned_placement": (_I, [_P, _I, _I]),
    "macsav_plan_set_first_solve_tolerance": (_I, [_P, _D]),
    "macsav_plan_set_launch_shape": (_I, [_P, _I]),
    "macsav_plan_autotune_launch_shapes": (_I, [_P, _I, C.POINTER(C.c_int), _P]),
    "macsav_transform32": (_I, [_P, _I, _I, _I, _I, _I, _P, _P, _P]),
    "macsav_transform32_autotune": (_I, [_P, _I, _I, _I, _I, C.POINTER(_I), C.POINTER(_D), C.POINTER(_D), _P]),
    "macsav_plan_cg_counters": (_I, [_P, _I, _P, _P, _P]),
    "macsav_stokes_log": (_I, [_P, _P, _D, _D, _I, _P, _P, _P, C.POINTER(_I), _P]),
    "macsav_step_embedded_norms": (_I, [_P, C.POINTER(_D)]),
    "macsav_integrate_adaptive": (_I, [_P, _I, _D, _D, _D, _D, _D, _P, _D, C.POINTER(StepControl), _P,
                                       C.POINTER(AdaptiveResult), C.POINTER(AdaptiveAttempt), _I, _P]),
    "macsav_channel_create": (_I, [C.POINTER(_P), _I, _I, _D, _D, _D, _I]),
    "macsav_channel_destroy": (None, [_P]),
    "macsav_channel_error": (C.c_char_p, [_P]),
    "macsav_channel_apply": (_I, [_P, _I, _P, _P, _I, _P]),
    "macsav_channel_combine": (_I, [_P, _I, C.POINTER(_D), C.POINTER(_P), _P, _LL, _P]),
    "macsav_channel_reduce": (_I, [_P, _P, _P, _LL, C.POINTER(_D), _P]),
    "macsav_channel_flow_rates": (_I, [_P, _P, _P, _P]),
    "macsav_channel_solve": (_I, [_P, _P, _I, _D, _D, _P, _P, C.POINTER(_D), C.POINTER(_D), C.POINTER(_I), _P]),
    "macsav_plan_create_members": (_I, [C.POINTER(_P), _I, _I, _D, _D, _I, _D, _D, _I, _I]),
    "macsav_plan_members": (_I, [_P]),
    "macsav_step_members_enqueue": (_I, [_P, _I, _D, _D, C.POINTER(_D), _D, _P, C.POINTER(_D), _P, _P, _P, _P, _P]),
    "macsav_step_members_finish": (_I, [_P, _P, C.POINTER(_D)]),
    "macsav_set_programmatic_launch": (_I, [_I]),
    "macsav_layout": (_I, [_P, _I, _P, _P, _P, _P]),
    "macsav_host_mapped": (_I, [_P, _LL, C.POINTER(_I)]),
    "macsav_copy_vectors": (_I, [_I, _P, _P, _P, _LL, _P]),
    "macsav_step_enqueue": (_I, [_P, _I, _D, _D, _D, _D, _P, _D, _P, _P, _P, _P, _P]),
    "macsav_step_finish": (_I, [_P, C.POINTER(StageRecord), C.POINTER(_D)]),
    "macsav_time_pass": (_I, [_P, _I, _I, C.POINTER(_D), C.POINTER(_D), _P]),
    "macsav_plan_set_refinement": (_I, [_P, _I, _D]),
}

_lib = None


def header_symbols() -> list[str]:
    """Function names declared in include/macsav.h."""
    text = HEADER.read_text()
    return sorted(set(re.findall(r"\b(macsav_[a-z0-9_]+)\s*\(", text)))


def load(path: pathlib.Path | None = None):
    """Load (once) and return the library; raises ImportError if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p.name} is not built: run __graft_entry__.build() (no CPU fallback exists)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def error_message(plan) -> str:
    msg = load().macsav_plan_error(plan)
    return msg.decode() if msg else ""


def check(code: int, plan) -> None:
    """Raise the reference's exception for a non-zero status code."""
    if code == OK:
        return
    msg = error_message(plan)
    if code in (ERR_VALUE,):
        raise ValueError(msg)
    if code in (ERR_CG, ERR_STOKES_GATE, ERR_STAGE_GATE, ERR_NEG_ENERGY, ERR_SCALAR):
        raise RuntimeError(msg)
    if code == ERR_UNSUPPORTED:
        raise ValueError(f"unsupported by the GB300 library: {msg}")
    raise MacsavError(msg or f"macsav error code {code}")
