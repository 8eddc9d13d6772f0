"""ctypes wrapper of the C oracle (nexus_oracle.c) -- TEST INFRASTRUCTURE.

Arrays are numpy uint64 in SEAL's layout ([size][limbs][N]).  Every method
names the SEAL routine it restates; the C file cites the lines.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "libnexus_oracle.so"
_lib = None

u64p = C.POINTER(C.c_uint64)
u32p = C.POINTER(C.c_uint32)


def build() -> Path:
    """Compile the oracle with its Makefile (gcc, a second or two)."""
    src = HERE / "nexus_oracle.c"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "libnexus_oracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        l = C.CDLL(str(LIB_PATH))
        l.or_ctx_create.restype = C.c_void_p
        l.or_ctx_create.argtypes = [C.c_int, u64p, C.c_int]
        l.or_ctx_destroy.argtypes = [C.c_void_p]
        l.or_ctx_root.restype = C.c_uint64
        l.or_ctx_root.argtypes = [C.c_void_p, C.c_int]
        l.or_ctx_root_powers.argtypes = [C.c_void_p, C.c_int, u64p, u64p]
        l.or_create_coeff_modulus.restype = C.c_int
        l.or_create_coeff_modulus.argtypes = [C.c_uint64, C.POINTER(C.c_int), C.c_int, u64p]
        l.or_minimal_primitive_root.restype = C.c_uint64
        l.or_minimal_primitive_root.argtypes = [C.c_uint64, C.c_uint64]
        l.or_ntt_batch.argtypes = [C.c_void_p, u64p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_int, C.c_int]
        l.or_ntt_lazy_limb.argtypes = [C.c_void_p, u64p, C.c_int]
        l.or_rescale_ntt.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p]
        l.or_drop_last_limb.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p]
        l.or_switch_key.argtypes = [C.c_void_p, u64p, C.c_int, u64p, u64p]
        l.or_relinearize.argtypes = [C.c_void_p, u64p, C.c_int, u64p, u64p]
        l.or_galois_table_ntt.argtypes = [C.c_int, C.c_uint32, u32p]
        l.or_galois_elt_from_step.restype = C.c_uint32
        l.or_galois_elt_from_step.argtypes = [C.c_int, C.c_int]
        l.or_apply_galois.argtypes = [C.c_void_p, u64p, C.c_int, C.c_uint32, u64p, u64p]
        l.or_ckks_multiply.argtypes = [C.c_void_p, u64p, u64p, C.c_int, u64p]
        l.or_multiply_plain.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p, u64p]
        l.or_add_sub.argtypes = [C.c_void_p, u64p, u64p, C.c_int, C.c_int, C.c_int, u64p]
        for f in ("or_mulmod", "or_invmod"):
            getattr(l, f).restype = C.c_uint64
            getattr(l, f).argtypes = [C.c_uint64, C.c_uint64, C.c_uint64][: 3 if f == "or_mulmod" else 2]
        l.or_encoder_create.restype = C.c_void_p
        l.or_encoder_create.argtypes = [C.c_int]
        l.or_encoder_destroy.argtypes = [C.c_void_p]
        l.or_encode.restype = C.c_int
        l.or_encode.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_double, C.c_int, u64p]
        l.or_encode_scalar.restype = C.c_int
        l.or_encode_scalar.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, u64p]
        l.or_multiply_scalar.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p, u64p]
        l.or_add_scalar.argtypes = [C.c_void_p, u64p, C.c_int, u64p, C.c_int, u64p]
        l.or_is_prime.restype = C.c_int
        l.or_is_prime.argtypes = [C.c_uint64]
        l.or_set_threads.argtypes = [C.c_int]
        l.or_get_threads.restype = C.c_int
        _lib = l
    return _lib


def set_threads(t: int) -> None:
    """Threads the oracle's key switch and rescale spread over (1: the caller only).
    The words do not depend on it."""
    lib().or_set_threads(int(t))


def get_threads() -> int:
    return int(lib().or_get_threads())


def _p(a: np.ndarray):
    assert a.dtype == np.uint64 and a.flags.c_contiguous
    return a.ctypes.data_as(u64p)


def create_coeff_modulus(n: int, bit_sizes) -> list[int]:
    """CoeffModulus::Create(n, bit_sizes) (SEAL modulus.cpp:143-184)."""
    bs = (C.c_int * len(bit_sizes))(*bit_sizes)
    out = np.zeros(len(bit_sizes), dtype=np.uint64)
    if lib().or_create_coeff_modulus(n, bs, len(bit_sizes), _p(out)) != 0:
        raise ValueError("failed to find enough qualifying primes")
    return [int(x) for x in out]


def minimal_primitive_root(degree: int, q: int) -> int:
    return int(lib().or_minimal_primitive_root(degree, q))


def galois_elt_from_step(log_n: int, step: int) -> int:
    return int(lib().or_galois_elt_from_step(log_n, step))


def galois_table_ntt(log_n: int, elt: int) -> np.ndarray:
    out = np.zeros(1 << log_n, dtype=np.uint32)
    lib().or_galois_table_ntt(log_n, elt, out.ctypes.data_as(u32p))
    return out


class OracleContext:
    """Per-prime NTT tables for primes q[0..k-1] (last = special prime)."""

    def __init__(self, log_n: int, moduli):
        self.log_n = int(log_n)
        self.n = 1 << self.log_n
        self.moduli = [int(q) for q in moduli]
        self.k = len(self.moduli)
        arr = np.array(self.moduli, dtype=np.uint64)
        self._h = lib().or_ctx_create(self.log_n, _p(arr), self.k)
        if not self._h:
            raise MemoryError("or_ctx_create failed")

    def __del__(self):
        if getattr(self, "_enc", None):
            lib().or_encoder_destroy(self._enc)
            self._enc = None
        if getattr(self, "_h", None):
            lib().or_ctx_destroy(self._h)
            self._h = None

    def root(self, j: int) -> int:
        return int(lib().or_ctx_root(self._h, j))

    def root_powers(self, j: int):
        a = np.zeros(self.n, dtype=np.uint64)
        b = np.zeros(self.n, dtype=np.uint64)
        lib().or_ctx_root_powers(self._h, j, _p(a), _p(b))
        return a, b

    # ntt_negacyclic_harvey / inverse_ntt_negacyclic_harvey (util/ntt.cpp:408-470)
    def ntt(self, a: np.ndarray, limb_begin: int, limb_end: int, inverse=False, threads=1) -> np.ndarray:
        a = np.ascontiguousarray(a, dtype=np.uint64).copy()
        limbs = limb_end - limb_begin
        n_polys = a.size // (limbs * self.n)
        lib().or_ntt_batch(self._h, _p(a), n_polys, limb_begin, limb_end, 1 if inverse else 0, threads)
        return a

    # RNSTool::divide_and_round_q_last_ntt_inplace (util/rns.cpp:830-905)
    def rescale(self, ct: np.ndarray) -> np.ndarray:
        size, limbs, n = ct.shape
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        out = np.zeros((size, limbs - 1, n), dtype=np.uint64)
        lib().or_rescale_ntt(self._h, _p(ct), size, limbs, _p(out))
        return out

    # Evaluator::switch_key_inplace (evaluator.cpp:2724-3022)
    def switch_key(self, ct: np.ndarray, target: np.ndarray, key: np.ndarray) -> np.ndarray:
        ct = np.ascontiguousarray(ct, dtype=np.uint64).copy()
        ell = ct.shape[1]
        target = np.ascontiguousarray(target, dtype=np.uint64)
        key = np.ascontiguousarray(key, dtype=np.uint64)
        assert key.shape[1:] == (2, self.k, self.n) and key.shape[0] >= ell
        lib().or_switch_key(self._h, _p(ct), ell, _p(target), _p(key))
        return ct

    # relinearize_internal (evaluator.cpp:1345-1400)
    def relinearize(self, ct3: np.ndarray, key: np.ndarray) -> np.ndarray:
        ell = ct3.shape[1]
        ct3 = np.ascontiguousarray(ct3, dtype=np.uint64)
        out = np.zeros((2, ell, self.n), dtype=np.uint64)
        lib().or_relinearize(self._h, _p(ct3), ell, _p(np.ascontiguousarray(key, dtype=np.uint64)), _p(out))
        return out

    # apply_galois_inplace (evaluator.cpp:2563-2665)
    def apply_galois(self, ct: np.ndarray, elt: int, key: np.ndarray) -> np.ndarray:
        ell = ct.shape[1]
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        out = np.zeros_like(ct)
        lib().or_apply_galois(self._h, _p(ct), ell, elt, _p(np.ascontiguousarray(key, dtype=np.uint64)), _p(out))
        return out

    # ckks_multiply (evaluator.cpp:770-850)
    def multiply(self, a: np.ndarray, b: np.ndarray) -> np.ndarray:
        ell = a.shape[1]
        out = np.zeros((3, ell, self.n), dtype=np.uint64)
        lib().or_ckks_multiply(self._h, _p(np.ascontiguousarray(a)), _p(np.ascontiguousarray(b)), ell, _p(out))
        return out

    # multiply_plain_ntt (evaluator.cpp:2336-2373)
    def multiply_plain(self, ct: np.ndarray, pt: np.ndarray) -> np.ndarray:
        size, ell, n = ct.shape
        out = np.zeros_like(ct)
        lib().or_multiply_plain(self._h, _p(np.ascontiguousarray(ct)), size, ell, _p(np.ascontiguousarray(pt)),
                                _p(out))
        return out

    # CKKSEncoder::encode (ckks.h:457-640) -> NTT-form [limbs][N]
    _ENC_ERR = {-1: "scale out of bounds", -2: "encoded values are too large", -3: "values_size is too large"}

    def encode(self, values, scale, limbs):
        if not hasattr(self, "_enc"):
            self._enc = lib().or_encoder_create(self.log_n)
        v = np.asarray(values)
        re = np.ascontiguousarray(v.real, dtype=np.float64)
        im = np.ascontiguousarray(v.imag, dtype=np.float64) if np.iscomplexobj(v) else None
        out = np.zeros((limbs, self.n), dtype=np.uint64)
        rc = lib().or_encode(self._h, self._enc, re.ctypes.data, None if im is None else im.ctypes.data, re.size,
                             float(scale), limbs, _p(out))
        if rc:
            raise ValueError(self._ENC_ERR[rc])
        return out

    # CKKSEncoder::encode(double) (ckks.cpp:75-205): per-limb residues
    def encode_scalar(self, value, scale, limbs):
        out = np.zeros(limbs, dtype=np.uint64)
        rc = lib().or_encode_scalar(self._h, float(value), float(scale), limbs, _p(out))
        if rc:
            raise ValueError({-1: "scale out of bounds", -2: "encoded value is too large"}[rc])
        return out

    def multiply_scalar(self, ct, per_limb):
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        out = np.zeros_like(ct)
        s = np.ascontiguousarray(per_limb, dtype=np.uint64)
        lib().or_multiply_scalar(self._h, _p(ct), ct.shape[0], ct.shape[1], _p(s), _p(out))
        return out

    def add_scalar(self, poly, per_limb, sub=False):
        poly = np.ascontiguousarray(poly, dtype=np.uint64)
        out = np.zeros_like(poly)
        s = np.ascontiguousarray(per_limb, dtype=np.uint64)
        lib().or_add_scalar(self._h, _p(poly), poly.shape[0], _p(s), 1 if sub else 0, _p(out))
        return out

    def add(self, a, b):
        out = np.zeros_like(a)
        lib().or_add_sub(self._h, _p(np.ascontiguousarray(a)), _p(np.ascontiguousarray(b)), a.shape[0], a.shape[1],
                         0, _p(out))
        return out

    def sub(self, a, b):
        out = np.zeros_like(a)
        lib().or_add_sub(self._h, _p(np.ascontiguousarray(a)), _p(np.ascontiguousarray(b)), a.shape[0], a.shape[1],
                         1, _p(out))
        return out


def random_residues(rng: np.random.Generator, shape, moduli_per_limb) -> np.ndarray:
    """Uniform residues in [0, q_l) for an array whose second-to-last axis is the limb axis."""
    q = np.array(moduli_per_limb, dtype=np.uint64).reshape((len(moduli_per_limb), 1))
    x = rng.integers(0, np.iinfo(np.uint64).max, size=shape, dtype=np.uint64, endpoint=True)
    return x % q


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)
