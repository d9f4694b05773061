"""GB300 library for the HAMS-MREL per-frequency boundary-integral path.

The compute lives in libhamsgpu.so (CUDA for sm_103a behind the C ABI of
include/hamsgpu.h); ``hamsgpu`` is its ctypes binding and ``meshgen`` builds
the synthetic benchmark meshes.  The directory name contains a hyphen, so
load it by path, e.g. with ``__graft_entry__.load_package()``.
"""
from . import hamsgpu, meshgen  # noqa: F401
