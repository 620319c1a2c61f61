"""GB300-native (sm_103a) MAC mr-SAV stage: the no-slip MAC hot path of
HaifengWang1031/MAC-mr-SAV-RK behind the reference's own API.

Public names mirror the reference: ``MACGrid``, ``TensorStokes`` (Stokes
backend), ``MACNavierStokes`` (model seam), ``make_scheme`` / ``scheme_info``
(fused GPU schemes); the model and the schemes plug into the reference's own
``integrate`` / ``integrate_adaptive``.  ``run_fixed`` / ``run_adaptive`` are
the package's device-resident loops for the fused schemes, and
``run_adaptive_device`` keeps the adaptive attempt loop itself on the device.  All compute runs
in ``libmacsav.so`` (include/macsav.h); importing the GPU classes without the
built library raises.
"""
from .grid import MACGrid, grid_of  # noqa: F401
from . import fields  # noqa: F401

from .core import DeviceArray, Stage, State, Trial, stage_diagnostics  # noqa: F401

__all__ = ["MACGrid", "grid_of", "fields", "State", "Stage", "Trial", "DeviceArray", "stage_diagnostics",
           "run_fixed", "run_adaptive", "run_adaptive_device", "StepControl", "FixedRun", "AdaptiveRun",
           "TensorStokes", "StokesResult", "Plan", "MACNavierStokes", "make_scheme", "scheme_info", "SCHEMES",
           "ChannelGrid", "ChannelModel", "ChannelOperators", "FFTStokes", "Ensemble", "ensemble_members",
           "shard_members", "UNet"]

_LAZY = {"TensorStokes": "stokes", "StokesResult": "stokes", "Plan": "stokes", "MACNavierStokes": "model",
         "make_scheme": "schemes", "scheme_info": "schemes", "SCHEMES": "schemes", "FusedScheme": "schemes",
         "ChannelGrid": "channel", "ChannelModel": "channel", "ChannelOperators": "channel", "FFTStokes": "channel",
         "Ensemble": "ensemble", "ensemble_members": "ensemble", "shard_members": "ensemble", "UNet": "learned",
         "run_fixed": "drive", "run_adaptive": "drive", "run_adaptive_device": "drive", "StepControl": "drive",
         "FixedRun": "drive",
         "AdaptiveRun": "drive"}


def __getattr__(name):
    # GPU-facing modules import torch and the CUDA library lazily.
    if name in _LAZY:
        from importlib import import_module
        return getattr(import_module(f"{__name__}.{_LAZY[name]}"), name)
    raise AttributeError(name)
