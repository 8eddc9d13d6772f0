"""Python handle over ``nexus_context`` (include/nexus_gb300.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


def create_coeff_modulus(poly_degree: int, bit_sizes) -> list[int]:
    """Primes chosen exactly as SEAL's CoeffModulus::Create chooses them."""
    bs = (C.c_int * len(bit_sizes))(*[int(b) for b in bit_sizes])
    out = (C.c_uint64 * len(bit_sizes))()
    check(lib().nexus_create_coeff_modulus(int(poly_degree), bs, len(bit_sizes), out), "create_coeff_modulus")
    return [int(x) for x in out]


class Context:
    """RNS context: data primes followed by the special prime."""

    def __init__(self, log_n: int, moduli):
        self.log_n = int(log_n)
        self.n = 1 << self.log_n
        self.moduli = [int(q) for q in moduli]
        arr = (C.c_uint64 * len(self.moduli))(*self.moduli)
        h = C.c_void_p()
        check(lib().nexus_context_create(self.log_n, arr, len(self.moduli), C.byref(h)), "nexus_context_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            lib().nexus_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def psi(self) -> np.ndarray:
        out = np.zeros(len(self.moduli), dtype=np.uint64)
        check(lib().nexus_context_get_psi(self._h, out.ctypes.data_as(C.POINTER(C.c_uint64))), "get_psi")
        return out

    # ---- NTT on device tensors ------------------------------------------
    def ntt_forward(self, t, limb_begin: int, limb_end: int, stream=None):
        """In-place forward NTT of a CUDA uint64 tensor shaped [..., limbs, N]."""
        n_polys = t.numel() // ((limb_end - limb_begin) * self.n)
        check(lib().nexus_ntt_forward(self._h, t.data_ptr(), n_polys, limb_begin, limb_end, _stream_ptr(stream)),
              "nexus_ntt_forward")

    def ntt_inverse(self, t, limb_begin: int, limb_end: int, stream=None):
        n_polys = t.numel() // ((limb_end - limb_begin) * self.n)
        check(lib().nexus_ntt_inverse(self._h, t.data_ptr(), n_polys, limb_begin, limb_end, _stream_ptr(stream)),
              "nexus_ntt_inverse")
