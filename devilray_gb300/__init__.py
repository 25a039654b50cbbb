"""GB300-native path-tracing core with DevilRay's interface.

``devilray_gb300.native`` binds the C ABI (include/devilray_gb300.h) of the
in-tree CUDA library; ``devilray_gb300.scenes`` builds the seeded synthetic
workloads.
"""
from . import build, native, scenes  # noqa: F401

__all__ = ["build", "native", "scenes"]
