"""CPU oracle for Rhyme's MUSCL-Hancock path (test infrastructure only).

Only tests/, __graft_entry__.smoke() (as the checker) and bench.py's CPU
baseline legs import this package. The CUDA library never uses it.
"""
from .pyoracle import *  # noqa: F401,F403
