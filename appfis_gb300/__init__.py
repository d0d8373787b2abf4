"""GB300-native APPFIS stencil engine.

The product is the C ABI library libappfis_gb.so (include/appfis_gb.h, sources in csrc/) and
the drop-in C++ headers in Appfis/ that keep the reference framework's API.  This Python
package only loads and calls that library (ctypes) and generates the seeded workloads; it has
no compute path of its own.
"""
from . import _lib
from ._lib import AppfisError, call, declared_symbols, lib, ptr

__all__ = ["AppfisError", "call", "declared_symbols", "lib", "ptr", "_lib"]
