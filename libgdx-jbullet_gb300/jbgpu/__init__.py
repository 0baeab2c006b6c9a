"""jbgpu: JBullet's per-step rigid-body pipeline on one GB300 (sm_103a).

The product is libjbgpu.so and its C ABI (include/jbgpu.h).  This package holds the
Python side of that boundary: the ctypes binding (lib.GpuWorld), a mirror of the
reference's world/body/shape API (dynamics), and seeded synthetic scenes (scenes).
"""
from . import _abi, scenes  # noqa: F401

__all__ = ["_abi", "scenes", "lib", "dynamics"]
