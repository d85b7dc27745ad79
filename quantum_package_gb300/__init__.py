"""GB300-native Davidson sigma path of Quantum Package (sigma = H.C, S^2.C).

The compute path is libqpgpu.so (CUDA, sm_103a) behind the C-ABI of
include/qpgpu.h; this package holds its Python mirror of the reference
interface and the seeded input generator.
"""
from ._lib import (ALGEBRA_FAST, ALGEBRA_FP64, ALGEBRA_TC, FF, FP32, FP64, KEYS_OFF, SIGMA_AUTO,  # noqa: F401
                   SIGMA_DIRECT, SIGMA_STORED, QPGPUError)

__all__ = ["FP32", "FP64", "QPGPUError"]
