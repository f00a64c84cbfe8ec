"""fastmc_gb300: GB300-native (sm_103a) GCMC trial-move energy path.

The hot path (pair energies over cell columns, Ewald k-space, Metropolis
and the structure-factor commit) runs as hand-written CUDA kernels
behind the C ABI in include/fastmc_gb300.h.  This package holds the build
script, the ctypes binding and a small Python API; see api.py.
"""
from ._lib import (FMC_PREC_FP32, FMC_PREC_FP64, FmcError, LIB_PATH, MOVE_NAMES,  # noqa: F401
                   load)
from .api import Batch, PlainEngine, System  # noqa: F401

__all__ = ["System", "PlainEngine", "Batch", "FMC_PREC_FP64", "FMC_PREC_FP32", "FmcError",
           "load", "LIB_PATH", "MOVE_NAMES"]
