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

__all__ = ["MACGrid", "grid_of", "fields", "TensorStokes", "StokesResult", "Plan"]


def __getattr__(name):
    # GPU-facing modules import torch and the CUDA library lazily.
    if name in ("TensorStokes", "StokesResult", "Plan"):
        from . import stokes
        return getattr(stokes, name)
    raise AttributeError(name)
