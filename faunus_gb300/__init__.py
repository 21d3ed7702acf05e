"""GB300-native Metropolis Monte Carlo energy hot path (Faunus drop-in).

The compute path is ``libfau_gpu.so`` (hand-written sm_103a CUDA behind the
C ABI of ``include/fau_gpu.h``); this package is its Python host API.
"""
from . import _capi
from ._capi import FauError
from .system import (Context, MoveGenerator, Sampler, System, SystemSpec, bjerrum_length, footprint,
                     group_cutoff, coulomb_scheme, kjmol_to_kt, move_descs, pressure_kt, splined, andrea_spline,
                     andrea_eval)

__all__ = ["Context", "Sampler", "System", "SystemSpec", "MoveGenerator", "FauError", "bjerrum_length",
           "kjmol_to_kt", "footprint", "group_cutoff", "coulomb_scheme", "move_descs", "pressure_kt",
           "splined", "andrea_spline", "andrea_eval", "_capi"]
