"""GB300-native GPIS ray-flight library (sparse-convolution-noise medium).

The compute path is libgpis_gb300.so (hand-written sm_103a CUDA kernels behind a
C ABI, include/gpis.h); this package holds its ctypes binding (abi), the
Tungsten-facing medium adapter (medium), seeded workloads and the build recipe.
"""
from . import abi  # noqa: F401
