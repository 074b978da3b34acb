"""GB300-native structured volume ray caster (sm_103a CUDA behind a C ABI).

The product is the shared library cpp_volume_rendering_gb300/_build/libcvr.so
(declared in include/cvr.h); this package holds its sources (csrc/), the
in-tree build (build.py) and a ctypes mirror of the ABI for Python callers.
"""
from . import abi  # noqa: F401

__all__ = ["abi"]
