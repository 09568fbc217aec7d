"""Square-Wheel world-rendering hot path on GB300: Python host binding and synthetic inputs.

The compute path is the CUDA library built from csrc/ (libswgpu.so, C ABI in include/swgpu.h).
"""
from . import abi  # noqa: F401
