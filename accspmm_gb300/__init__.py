"""GB300 METCF SpMM: a drop-in for the AccSpMM path behind a C ABI.

The product is libaccspmm.so (include/accspmm.h) and the `mma` command; this
package holds their sources (csrc/), the build recipe (build.py), ctypes
bindings (capi.py), a host-side mirror of the reference's C++ calls (api.py)
and seeded workload generators (synth.py).
"""
from . import capi  # noqa: F401

__all__ = ["capi", "api", "synth", "build"]
