"""GB300-native FCIQMC iteration engine: a drop-in for NECI's PerformFCIMCycPar.

The compute path is the CUDA library ``_build/libneci_gpu.so`` (sources in
``csrc/``, C ABI in ``include/neci_gpu.h``).  This package is the host side
that NECI's Fortran keeps: system set-up (``systems``), the ctypes view of
the C ABI (``capi``, ``engine``), the FciMCPar loop with the shift update
(``fcimc``) and the blocking analysis (``analysis``).  Importing it does not
build or load the library; ``capi.load()`` does, and fails loudly if the
library is missing.
"""
from . import capi  # noqa: F401

__all__ = ["capi", "build", "engine", "fcimc", "systems", "analysis"]
