"""GB300-native wavefront path tracer with path guiding.

The compute lives in libpgx.so (CUDA, sm_103a) behind the C ABI declared in
include/pgx.h; this package holds the ctypes binding (``abi``), the Python
mirror of the reference's Scene/RayTracer interface (``api``), the seeded
procedural scenes the workloads use (``scenes``) and the build recipe
(``build``).
"""
from . import abi, scenes  # noqa: F401

__all__ = ["abi", "scenes", "api", "build"]
