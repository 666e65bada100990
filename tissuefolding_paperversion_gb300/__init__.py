"""GB300-native implicit prism time step of TissueFolding.

The product is ``_lib/libtfgpu.so`` (C ABI in ``include/tf_gpu.h``): a
device-resident Newton-Raphson step -- prism residual and 18x18 tangent,
block-sparse assembly, boundary conditions, external viscosity and an FP64
Krylov solve -- written as hand-written CUDA for sm_103a with a C++ host.
``api`` binds it with ctypes; ``mesh`` builds seeded workloads.
"""
from . import build, mesh  # noqa: F401

__all__ = ["api", "build", "mesh"]
