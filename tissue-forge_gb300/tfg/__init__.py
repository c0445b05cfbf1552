"""tfg: GB300-native engine for Tissue Forge's per-step particle path.

The compute path is libtfg.so (hand-written CUDA for sm_103a behind a C ABI,
include/tfg.h).  This package is a thin ctypes layer over it that mirrors the
reference's Potential / Fluxes / Bond / engine objects for Python callers.
"""
from . import abi, configs  # noqa: F401
from ._lib import lib, lib_path  # noqa: F401
from .potentials import Potential  # noqa: F401
from .engine import Batch, Engine, Sim, TfgError  # noqa: F401
