"""GB300-native (sm_103a) implementation of M3TET_SPH's time-step hot path.

The compute lives in the in-tree CUDA library ``libm3sph.so`` (C ABI: include/m3sph.h);
this package holds the host-side set-up (mesh hierarchy, synthetic workloads) and the Python
mirror of the reference's MATLAB interface.
"""
from . import mesh, workloads  # noqa: F401

__all__ = ["mesh", "workloads"]
