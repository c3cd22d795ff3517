"""GB300-native (sm_103a) DiskDyn dynamical and imaging path.

The compute lives in libddx.so (CUDA kernels + C ABI, include/diskdyn_gb300.h); this
package is its Python host interface.  Importing it does not load the library; the
first Engine does, and raises if the library was not built.
"""
from . import abi, synth  # noqa: F401
from .abi import (DDX_MODE_FIXED, DDX_MODE_REFERENCE, DDX_PREC_FP64, DDX_PREC_MIXED,  # noqa: F401
                  DDXError)

__all__ = ["abi", "synth", "DDX_PREC_FP64", "DDX_PREC_MIXED", "DDX_MODE_FIXED",
           "DDX_MODE_REFERENCE", "DDXError"]
