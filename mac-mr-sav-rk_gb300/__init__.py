"""GB300-native (sm_103a) MAC mr-SAV stage: the no-slip MAC hot path of
HaifengWang1031/MAC-mr-SAV-RK behind the reference's own API.

Public names mirror the reference: ``MACGrid``, ``TensorStokes`` (Stokes
backend), ``MACNavierStokes`` (model seam), ``make_scheme`` / ``scheme_info``
(fused GPU schemes), ``integrate`` (fixed-step driver).  All compute runs in
``libmacsav.so`` (include/macsav.h); importing the GPU classes without the
built library raises.
"""
from .grid import MACGrid, grid_of  # noqa: F401
from . import fields  # noqa: F401

from .core import DeviceArray, Stage, State, Trial, stage_diagnostics  # noqa: F401
from .integrate import Result, integrate, nearest_node_indices, schedule_nodes, step_sizes  # noqa: F401

__all__ = ["MACGrid", "grid_of", "fields", "State", "Stage", "Trial", "DeviceArray", "stage_diagnostics",
           "Result", "integrate", "step_sizes", "schedule_nodes", "nearest_node_indices",
           "TensorStokes", "StokesResult", "Plan", "MACNavierStokes", "make_scheme", "scheme_info", "SCHEMES",
           "ChannelGrid", "ChannelModel", "ChannelOperators", "FFTStokes", "Ensemble", "ensemble_members",
           "shard_members", "UNet", "integrate_adaptive", "IController", "PIController"]

_LAZY = {"TensorStokes": "stokes", "StokesResult": "stokes", "Plan": "stokes", "MACNavierStokes": "model",
         "make_scheme": "schemes", "scheme_info": "schemes", "SCHEMES": "schemes", "FusedScheme": "schemes",
         "ChannelGrid": "channel", "ChannelModel": "channel", "ChannelOperators": "channel", "FFTStokes": "channel",
         "Ensemble": "ensemble", "ensemble_members": "ensemble", "shard_members": "ensemble", "UNet": "learned",
         "integrate_adaptive": "adaptivity", "IController": "adaptivity", "PIController": "adaptivity"}


def __getattr__(name):
    # GPU-facing modules import torch and the CUDA library lazily.
    if name in _LAZY:
        from importlib import import_module
        return getattr(import_module(f"{__name__}.{_LAZY[name]}"), name)
    raise AttributeError(name)
