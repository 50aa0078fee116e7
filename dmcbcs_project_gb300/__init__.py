"""GB300 (sm_103a) implementation of the DMCBS walker hot path.

The compute path is the CUDA library ``libdmcbcs_gb300.so`` built from
``csrc/`` (C ABI in ``include/dmcbcs_gpu.h``).  This package holds its
build script, the ctypes binding, the reader of the reference's input deck
and the synthetic benchmark workloads.
"""
from . import abi, configs, deck  # noqa: F401

__all__ = ["abi", "configs", "deck", "capi", "build"]
