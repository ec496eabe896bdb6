"""GB300-native (sm_103a) engine for Pachyderm's stochastic split ray tracer.

The compute path is libpach_gpu.so (hand-written CUDA + a C ABI, include/pach_gpu.h).  Python
reaches it through ctypes: ``tracer`` (array-level API), ``simulation`` (the reference's
SplitRayTracer / Polygon_Scene / Receiver_Bank API) and ``rooms`` (seeded benchmark rooms).
"""
from . import rooms  # noqa: F401

__all__ = ["rooms", "tracer", "simulation", "build"]
