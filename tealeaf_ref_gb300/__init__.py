"""GB300-native (sm_103a) TeaLeaf implicit heat-diffusion solve.

The compute path is libtealeaf_gb300.so (hand-written CUDA behind the C ABI in
include/tealeaf_gb300.h); this package holds its build recipe, the ctypes binding
(``native``) and the input-deck reader/writer (``deck``).
"""
from . import deck  # noqa: F401

__all__ = ["deck", "native", "build"]
__version__ = "0.1.0"
