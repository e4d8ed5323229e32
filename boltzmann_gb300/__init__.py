"""GB300 (sm_103a) electron PIC-MCC hot path of jfabell/boltzmann.

Hand-written CUDA kernels behind the C ABI in include/bz.h (libbz.so), driven from
Python through ctypes. PyTorch only owns device memory and supplies the stream.
"""
from ._lib import BzError, BzLibraryError, load  # noqa: F401

__all__ = ["BzError", "BzLibraryError", "load"]
