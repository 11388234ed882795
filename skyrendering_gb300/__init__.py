"""skyrendering_gb300 — GB300-native atmosphere LUTs, procedural volumetric
clouds and voxel path tracing behind the C ABI of include/skyr.h.

The compute path is libskyr.so (hand-written sm_103a kernels); this package is
the host-side mirror of the reference's class interface and the ctypes binding.
"""
from . import _abi  # noqa: F401
from ._abi import SkyrError, lib  # noqa: F401

__all__ = ["SkyrError", "lib"]
