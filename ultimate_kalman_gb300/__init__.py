"""GB300-native parallel Kalman smoothers (odd-even and associative) behind
UltimateKalman's C API.

The product is the C-ABI library ``libukgpu.so`` (include/kalman.h,
include/kalman_gpu.h) with hand-written CUDA kernels for sm_103a, built by
``ultimate_kalman_gb300.build``.  ``native`` binds it with ctypes; ``problem``
holds the packed problem type and the synthetic workload generators.
"""
from . import problem  # noqa: F401

__all__ = ["problem", "native", "build"]
