"""GB300-native imaging-FCS correlation-and-fit engine.

The compute lives in the CUDA library libimfcs_gb300.so (csrc/, C ABI in
include/imfcs_gb300.h).  `engine` is the whole-path API (uint16 stack ->
ACF, blocked variance, LM/GLS fits, Bayes, diffusion law); `gpufit_imfcs`
mirrors the plugin's GpufitImFCS JNI class for the reference-facing calls.
"""
__version__ = "0.1.0"

from . import _lib  # noqa: F401
