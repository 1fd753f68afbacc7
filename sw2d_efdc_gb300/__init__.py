"""GB300-native SW2D explicit 2-D overland shallow-water step.

The compute path is the CUDA library ``_lib/libsw2d.so`` (sources in
``csrc/``, C ABI in ``include/sw2d.h``); ``api`` is its ctypes mirror and
``synth`` the seeded input generators.
"""
from . import api, synth  # noqa: F401

__all__ = ["api", "synth"]
