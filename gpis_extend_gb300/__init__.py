"""GB300-native GPIS ray-flight library (sparse-convolution-noise medium).

The compute path is libgpis_gb300.so (hand-written sm_103a CUDA kernels behind a
C ABI, include/gpis.h).  The Tungsten-facing medium adapter (sampleDistance /
transmittance state machines and the scene-JSON keys) is C++ inside that
library (csrc/medium_adapter.cpp, csrc/medium_json.cpp).  This package holds
its ctypes binding (abi), contexts over device memory (runtime), the learned
proposal's host side (proposal), the autotuner (autotune), seeded workloads and
the build recipe (build).
"""
from . import abi  # noqa: F401
