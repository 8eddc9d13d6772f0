"""nexus_gb300: a GB300-native CKKS evaluation engine for NEXUS's
encrypted-inference hot path.

The compute path is hand-written sm_103a CUDA behind the C ABI declared in
``include/nexus_gb300.h``; this package holds the build script and a thin
ctypes layer used by the tests and the benchmark.
"""
from ._lib import NexusError, check, lib  # noqa: F401
from .context import (SEAL_CBD, SEAL_SPARSE_TERNARY, SEAL_TERNARY, SEAL_UNIFORM, Context,  # noqa: F401
                      butterfly_rate, create_coeff_modulus, kernel_launches, memory_info, memory_trim, seal_prng_bytes,
                      seal_sample_poly, seal_seed,
                      TENSOR_BF16, TENSOR_E4M3, tensor_rate, tensor_tile)
