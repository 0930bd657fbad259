"""GB300-native partial-assembly H1 operator path (MFEM-compatible).

The compute path is libgbpa.so (CUDA, sm_103a), bound through its C ABI in
_lib.py; pa.py mirrors the reference's PA interface on top of it; fem.py holds
the host-side discretisation data (meshes, spaces, basis tables) and loads no
native code. The CUDA library is loaded on first use -- `mfem_gb300.lib`, or
`pa.Device()` -- and that first use raises if the library has not been built:
there is no CPU fallback.
"""

__all__ = ["lib"]


def __getattr__(name):
    if name == "lib":
        from . import _lib
        return _lib.load()
    raise AttributeError(f"module {__name__!r} has no attribute {name!r}")
