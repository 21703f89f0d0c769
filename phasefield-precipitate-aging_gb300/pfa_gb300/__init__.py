"""pfa_gb300: GB300-native explicit step of the KKS Cr-Nb-Ni precipitate-aging model.

The compute path is libpfa_gb300.so (CUDA, sm_103a) behind the reference's
own interface; this package holds its ctypes binding (lib), the seeded
initial conditions of the benchmark workloads (ic), and the build recipe
(build).
"""
from . import ic  # noqa: F401

__all__ = ["ic", "lib", "build"]
