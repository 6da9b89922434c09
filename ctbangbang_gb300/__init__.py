"""ctbangbang_gb300 -- GB300-native helical weighted-FBP reconstruction.

The compute path is libctbb_gb300.so (hand-written sm_103a CUDA behind the C
ABI of include/ctbb_gb300.h).  This package holds the Python side of that ABI:
ctypes mirrors of the reference's boundary structs (structs), the library
loader (lib), and scan descriptions / planning / synthetic phantoms (scans).
"""
from . import structs  # noqa: F401
from .lib import CtbbError, call, check, load  # noqa: F401

__all__ = ["structs", "lib", "scans", "CtbbError", "call", "check", "load"]
