"""GB300-native EVP-FFT solver step of the Voce crystal-plasticity code.

The compute path is libvoce_gpu.so (hand-written sm_103a CUDA behind the C
ABI in include/voce_gpu.h); this package holds its build recipe
(``build``), the ctypes mirror of the C ABI (``capi``) and generators of
synthetic inputs in the reference's file formats (``synth``).
"""
from . import synth  # noqa: F401

__all__ = ["synth", "capi", "build"]
