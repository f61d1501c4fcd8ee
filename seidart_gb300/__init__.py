"""seidart_gb300: GB300 (sm_103a) FDTD time-stepping backend for SeidarT.

The CUDA library (libseidart_gb300.so, C ABI in include/seidart_gb300.h) runs
the seismic2 / seismic25 / electromag2 / electromag25 solvers of the
reference's legacy Fortran (legacy/fortran/seismicfdtd.f95,
legacy/fortran/electromagfdtd.f95) on the GPU in FP32, with FP64 host-side
coefficients.  This package is the Python host side.
"""
from ._lib import ELECTROMAG2, ELECTROMAG25, ELECTROMAG2C, SEISMIC2, SEISMIC25, KIND_NAMES, KIND_BY_NAME  # noqa: F401
from ._lib import LibraryMissingError, SfdError, UnstableError  # noqa: F401

__all__ = ["SEISMIC2", "SEISMIC25", "ELECTROMAG2", "ELECTROMAG25", "ELECTROMAG2C", "KIND_NAMES", "KIND_BY_NAME",
           "LibraryMissingError", "SfdError", "UnstableError"]
