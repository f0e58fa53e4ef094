"""hipacc_gb300: GB300 (sm_103a) kernels for the image-processing hot path of
Hipacc's generated code, behind a C ABI (include/hipacc_gb300.h).

``hipacc_gb300.build.build()`` compiles libhipacc_gb300.so in-tree;
``hipacc_gb300.api`` drives it from torch CUDA tensors.  The C++ host surface
(Image, Accessor, BoundaryCondition, Mask, Domain, IterationSpace, Kernel,
Pyramid, traverse, hipacc* runtime calls) is include/hipacc_gb300/hipacc.hpp.
"""
from . import _lib  # noqa: F401

__all__ = ["api", "build"]
