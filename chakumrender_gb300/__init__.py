"""chakumrender_gb300 — GB300 (sm_103a) implementation of ChakumRender's path-tracing hot path.

The product is libckr.so and its C ABI (include/ckr.h).  `ckr` is the ctypes binding.
"""
from . import ckr  # noqa: F401

__all__ = ["ckr"]
