"""tracetransform_gb300 -- the trace transform's sinogram + circus path on GB300.

A drop-in for maleadt/tracetransform's C++ getSinograms / getCircusFunctions /
Transformer: hand-written sm_103a CUDA kernels behind the C ABI of
include/tracetransform.h (libtt_gb300.so), with this package as the Python
host side.  Build the library with ``python -m tracetransform_gb300.build``.
"""
from . import api
from .api import (PFunctional, PFunctionalWrapper, Plan, TFunctional, TFunctionalWrapper,
                  Transformer, ValidationError, angles_from_step, getCircusFunctions,
                  getSinograms, gray2mat, mat2gray, nearest_orthonormal_sinogram, ortho_size,
                  pad, pad_geometry, readnetpbm, resize, rotate, transform_batch, writecsv,
                  writepgm, zscore)

__all__ = [
    "PFunctional", "PFunctionalWrapper", "Plan", "TFunctional", "TFunctionalWrapper",
    "Transformer", "ValidationError", "angles_from_step", "getCircusFunctions", "getSinograms",
    "gray2mat", "mat2gray", "nearest_orthonormal_sinogram", "ortho_size", "pad", "pad_geometry",
    "readnetpbm", "resize", "rotate", "transform_batch", "writecsv", "writepgm", "zscore",
]
__version__ = "0.1.0"
