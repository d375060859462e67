"""dgcuda_gb300 -- GB300-native 2D discontinuous-Galerkin RHS and time-step core.

The compute path is the native library ``_lib/libdgx.so`` (hand-written CUDA for
sm_103a behind the C ABI of ``include/dgx.h``); this package holds the mesh
generator and thin ctypes handles used by tests and benchmarks.
"""
from . import mesh  # noqa: F401
from ._ffi import (ADVECTION, EULER, FLUX_CENTRAL, FLUX_LLF, FP32, FP32_BF16X3, FP64,  # noqa: F401
                   IC_CONSTANT, IC_DENSITY_WAVE, IC_GAUSSIAN, IC_POLY, IC_VORTEX, DgxError)

__all__ = ["mesh", "ADVECTION", "EULER", "FLUX_CENTRAL", "FLUX_LLF", "FP32", "FP32_BF16X3",
           "FP64", "IC_CONSTANT", "IC_DENSITY_WAVE", "IC_GAUSSIAN", "IC_POLY", "IC_VORTEX",
           "DgxError"]
