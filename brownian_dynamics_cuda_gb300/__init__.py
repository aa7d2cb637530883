"""GB300-native Brownian-dynamics step for the mesoscale chromatin fiber.

The compute path is libbdgb300.so (hand-written sm_103a CUDA behind the C
ABI in include/bd_capi.h); this package holds its build driver, the ctypes
binding and the synthetic-fiber generator.
"""
from .capi import (BD_OK, LOG_CR, LOG_LIBM, NOISE_CHOLESKY, NOISE_KRYLOV, PREC_FP64, PREC_MIXED, BDError, Batch, Context, DevNoise, Fiber, Noise, LIB_PATH,  # noqa: F401
                   load_library)

__version__ = "0.1.0"
