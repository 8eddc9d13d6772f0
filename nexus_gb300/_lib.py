"""ctypes binding of libnexus_gb300.so (the C ABI in include/nexus_gb300.h).

The shared library is built in-tree by :mod:`nexus_gb300.build`.  Loading
fails loudly when it is missing: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libnexus_gb300.so"
_lib = None

u64p = C.POINTER(C.c_uint64)

# (name, restype, argtypes) of every exported entry point
SIGNATURES = [
    ("nexus_last_error", C.c_char_p, []),
    ("nexus_kernel_launches", C.c_uint64, []),
    ("nexus_memory_info", C.c_int, [C.POINTER(C.c_uint64)] * 4),
    ("nexus_memory_trim", C.c_int, []),
    ("nexus_create_coeff_modulus", C.c_int, [C.c_uint64, C.POINTER(C.c_int), C.c_int, u64p]),
    ("nexus_context_create", C.c_int, [C.c_int, u64p, C.c_int, C.POINTER(C.c_void_p)]),
    ("nexus_context_destroy", C.c_int, [C.c_void_p]),
    ("nexus_context_get_psi", C.c_int, [C.c_void_p, u64p]),
    ("nexus_ntt_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int, C.c_int, C.c_void_p]),
    ("nexus_ntt_inverse", C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int, C.c_int, C.c_void_p]),
    ("nexus_ntt_timing_begin", C.c_int, [C.c_void_p]),
    ("nexus_ntt_timing_end", C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_uint64),
                                       C.POINTER(C.c_uint64)]),
    ("nexus_multiply", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_rescale", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_switch_key", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_switch_key_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                         C.c_void_p]),
    ("nexus_switch_key_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_relinearize", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_apply_galois", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_galois_elt_from_step", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_uint32)]),
    ("nexus_add", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_sub", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_negate", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_keygen_secret", C.c_int, [C.c_void_p, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_keygen_relin", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint64, C.c_void_p, C.c_void_p]),
    ("nexus_keygen_galois", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint64, C.c_void_p, C.c_void_p]),
    ("nexus_encrypt_symmetric", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_uint64, C.c_void_p, C.c_void_p]),
    ("nexus_decrypt", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_seal_prng_bytes", C.c_int, [u64p, C.c_uint64, C.c_size_t, C.c_void_p]),
    ("nexus_seal_sample_poly", C.c_int, [u64p, C.c_uint64, C.c_int, C.c_int, u64p, C.c_int, C.c_int, u64p]),
    ("nexus_seal_keygen_secret", C.c_int, [C.c_void_p, u64p, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_seal_keygen_public", C.c_int, [C.c_void_p, u64p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_seal_keygen_relin", C.c_int, [C.c_void_p, u64p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_seal_keygen_galois", C.c_int, [C.c_void_p, u64p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p]),
    ("nexus_seal_encrypt", C.c_int, [C.c_void_p, u64p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_seal_encrypt_symmetric", C.c_int,
     [C.c_void_p, u64p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_encode", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_double, C.c_int, C.c_void_p,
                               C.c_void_p]),
    ("nexus_encode_scalar", C.c_int, [C.c_void_p, C.c_double, C.c_double, C.c_int, u64p]),
    ("nexus_multiply_scalar", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, u64p, C.c_void_p, C.c_void_p]),
    ("nexus_decode", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_void_p, C.c_void_p, C.c_size_t,
                               C.c_size_t, C.c_void_p]),
    ("nexus_evaluator_create", C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("nexus_evaluator_destroy", C.c_int, [C.c_void_p]),
    ("nexus_evaluator_add_galois_key", C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    ("nexus_ciphertext_create", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("nexus_ciphertext_destroy", C.c_int, [C.c_void_p]),
    ("nexus_ciphertext_load", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p]),
    ("nexus_ciphertext_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double),
                                        C.POINTER(C.c_void_p)]),
    ("nexus_ciphertext_store", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_gelu", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_softmax", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_layer_norm", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_ckks_op", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p]),
    ("nexus_encode_coefficients", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_size_t, C.c_double, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_gelu_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_softmax_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("nexus_layer_norm_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("nexus_ckks_op_batch", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_double,
                                      C.c_void_p]),
    ("nexus_mm_power_of_x", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_mm_expand", C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]),
    ("nexus_matrix_mul", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_int,
                                   C.c_double, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_bootstrapper_create", C.c_int, [C.c_void_p, C.c_long, C.c_long, C.c_long, C.c_long, C.c_double,
                                            C.c_long, C.c_long, C.c_long, C.c_long, C.POINTER(C.c_void_p)]),
    ("nexus_bootstrapper_destroy", C.c_int, [C.c_void_p]),
    ("nexus_bootstrapper_prepare_mod_polynomial", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int),
                                                            C.POINTER(C.c_double), C.c_double]),
    ("nexus_bootstrapper_set_inverse_polynomial", C.c_int,
     [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    ("nexus_bootstrapper_add_rot_steps", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]),
    ("nexus_bootstrapper_generate_lt", C.c_int, [C.c_void_p]),
    ("nexus_lt_coefficients_3", C.c_int, [C.c_int, C.c_int, C.c_long, C.c_int, C.c_void_p, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int)]),
    ("nexus_bootstrap", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_argmax", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_bootstrap_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_bootstrap_real_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_bootstrapper_stage", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_rotate_vector_many", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_rotate_vector_many_batch", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    ("nexus_argmax_batch", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("nexus_evaluator_set_hoisting", C.c_int, [C.c_void_p, C.c_int]),
    ("nexus_bootstrapper_stage_batch", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                                 C.c_void_p]),
    ("nexus_bootstrapper_cached_plaintexts", C.c_int, [C.c_void_p, u64p]),
    ("nexus_seal_ciphertext_save", C.c_int, [u64p, C.c_int, C.c_int, C.c_int, C.c_double, u64p, C.c_int,
                                             C.c_void_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    ("nexus_seal_ciphertext_load", C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(C.c_int),
                                             C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double), u64p,
                                             C.POINTER(C.c_int)]),
    ("nexus_plain_op", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_autotune", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_double)]),
    ("nexus_set_tuning", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("nexus_get_tuning", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("nexus_set_ntt_form", C.c_int, [C.c_void_p, C.c_int]),
    ("nexus_get_ntt_form", C.c_int, [C.c_void_p, C.c_void_p]),
    ("nexus_butterfly_rate", C.c_int,
     [C.c_int, C.c_uint64, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("nexus_graph_capture_begin", C.c_int, [C.c_void_p]),
    ("nexus_graph_capture_end", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("nexus_graph_launch", C.c_int, [C.c_void_p, C.c_void_p]),
    ("nexus_graph_info", C.c_int, [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                                   C.POINTER(C.c_size_t)]),
    ("nexus_graph_destroy", C.c_int, [C.c_void_p]),
    ("nexus_tensor_rate", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("nexus_tensor_tile", C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("nexus_bert_layer_create", C.c_int,
     [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
      C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_void_p)]),
    ("nexus_bert_layer_destroy", C.c_int, [C.c_void_p]),
    ("nexus_bert_layer_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), u64p]),
    ("nexus_bert_layer_rotation_steps", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int]),
    ("nexus_bert_layer_forward", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    ("nexus_bert_layer_stage", C.c_int,
     [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int]),
    ("nexus_bert_layer_set_timing", C.c_int, [C.c_void_p, C.c_int]),
    ("nexus_bert_layer_set_boot_pack", C.c_int, [C.c_void_p, C.c_int]),
    ("nexus_bert_layer_set_token_fold", C.c_int, [C.c_void_p, C.c_int]),
    ("nexus_bert_layer_stage_times", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.c_char_p,
                                               C.c_size_t, C.POINTER(C.c_int), C.c_int]),
]


class NexusError(RuntimeError):
    pass


def lib():
    """Return the loaded library, loading it on first use."""
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise NexusError(
                f"{_LIB_PATH} is missing: build it with `python -m nexus_gb300.build` "
                "(the engine has no CPU fallback)")
        l = C.CDLL(str(_LIB_PATH))
        for name, res, args in SIGNATURES:
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


def check(status: int, what: str = "") -> None:
    if status != 0:
        msg = lib().nexus_last_error().decode(errors="replace")
        raise NexusError(f"{what}: {msg}" if what else msg)
