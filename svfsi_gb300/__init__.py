"""GB300-native implicit-step engine for svFSI-style finite-element solves.

The compute path is libgsls.so (hand-written CUDA for sm_103a behind a C
ABI, include/gsls.h); this package holds its build script, the ctypes
binding, the svFSILS-shaped host interface and synthetic problem builders.
"""
__all__ = ["build", "fsils", "meshgen", "problems"]
