"""GB300-native MUSCL-Hancock hydro step for Rhyme SAMR boxes.

The product is the C-ABI library librhyme_gpu.so (include/rhyme_gpu.h),
built from rhyme_gb300/csrc for sm_103a. This package holds its build
recipe, a ctypes binding that mirrors the reference's Fortran module
interfaces, and seeded initial-condition generators.
"""
from . import params  # noqa: F401
