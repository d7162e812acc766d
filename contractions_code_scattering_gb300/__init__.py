"""GB300-native distillation contraction engine (rho, pi-pi, sigma, rho-pipi, sigma-pipi).

The compute path is libctr.so: hand-written sm_103a CUDA behind the C ABI of
include/ctr.h.  This package holds its build script, the ctypes binding, the
Python mirror of the reference launchers (api) and the synthetic-data
generators (synth).
"""

from ._lib import CtrError, ENGINE_FP64, ENGINE_SPLIT, lib, check  # noqa: F401
from ._build import build  # noqa: F401

__all__ = ["CtrError", "ENGINE_FP64", "ENGINE_SPLIT", "lib", "check", "build"]
