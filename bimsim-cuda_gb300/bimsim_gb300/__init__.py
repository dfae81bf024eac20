"""Host-side Python interface of the GB300 near-field-to-detector library.

The compute path is the CUDA library libbimsim_gb300.so (C ABI in
include/bimsim_gb300.h); this package only loads it with ctypes and moves
buffers.  There is no CPU fallback: every call fails if the library or a GPU
is missing.
"""
from .abi import (BS_FIELD_INCIDENT, BS_FIELD_TOTAL, BS_IMG_ABSORBANCE, BS_IMG_INCIDENT, BS_IMG_INTENSITY,
                  BS_IMG_TRANSMITTANCE, BS_PREC_FP64, BS_PREC_MIXED, Info, Params, Sphere, Stats, make_params,
                  sphere_array)
from .lib import BimsimError, Context, Server, estimate_bytes, library, library_path

__all__ = ["BS_FIELD_INCIDENT", "BS_FIELD_TOTAL", "BS_IMG_ABSORBANCE", "BS_IMG_INCIDENT", "BS_IMG_INTENSITY",
           "BS_IMG_TRANSMITTANCE", "BS_PREC_FP64", "BS_PREC_MIXED", "BimsimError", "Context", "Info", "Params",
           "Server", "Sphere", "Stats", "estimate_bytes", "library", "library_path", "make_params", "sphere_array"]
