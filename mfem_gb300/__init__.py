"""GB300-native partial-assembly H1 operator path (MFEM-compatible).

The compute path is libgbpa.so (CUDA, sm_103a), bound through its C ABI in
_lib.py; pa.py mirrors the reference's PA interface on top of it; fem.py holds
the host-side discretisation data. Importing the package loads the CUDA
library and raises if it has not been built.
"""
from . import _lib

lib = _lib.load()

__all__ = ["lib"]
