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


def _u64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_uint64))


def seal_seed(seed) -> np.ndarray:
    """SEAL's prng_seed_type: 8 words; an int sets word 0 and leaves the rest zero."""
    if isinstance(seed, (int, np.integer)):
        w = np.zeros(8, dtype=np.uint64)
        w[0] = int(seed)
        return w
    w = np.ascontiguousarray(seed, dtype=np.uint64)
    if w.shape != (8,):
        raise ValueError("a SEAL seed is 8 64-bit words")
    return w


def seal_prng_bytes(seed, offset: int, n: int) -> bytes:
    """Bytes [offset, offset + n) of SEAL's Blake2xbPRNG stream for `seed` (host only)."""
    out = (C.c_uint8 * max(1, n))()
    check(lib().nexus_seal_prng_bytes(_u64p(seal_seed(seed)), int(offset), int(n), out), "nexus_seal_prng_bytes")
    return bytes(out)[:n]


SEAL_TERNARY, SEAL_SPARSE_TERNARY, SEAL_CBD, SEAL_UNIFORM = 0, 1, 2, 3


def seal_sample_poly(seed, kind: int, log_n: int, moduli, hamming_weight: int = 0, offset: int = 0) -> np.ndarray:
    """One of SEAL's samplers (util/rlwe.cpp) on a fresh stream: residues [k][2^log_n] (host only)."""
    q = np.ascontiguousarray([int(x) for x in moduli], dtype=np.uint64)
    out = np.zeros((q.size, 1 << log_n), dtype=np.uint64)
    check(lib().nexus_seal_sample_poly(_u64p(seal_seed(seed)), int(offset), int(kind), int(log_n), _u64p(q), q.size,
                                       int(hamming_weight), _u64p(out)), "nexus_seal_sample_poly")
    return out


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

    # ---- ciphertext arithmetic on device tensors (SEAL layout) -----------
    def multiply(self, a, b, out3, stream=None):
        check(lib().nexus_multiply(self._h, a.data_ptr(), b.data_ptr(), a.shape[-2], out3.data_ptr(),
                                   _stream_ptr(stream)), "nexus_multiply")

    def rescale(self, ct, out, stream=None):
        size, limbs = ct.shape[0], ct.shape[1]
        check(lib().nexus_rescale(self._h, ct.data_ptr(), size, limbs, out.data_ptr(), _stream_ptr(stream)),
              "nexus_rescale")

    def switch_key(self, ct, target, key, stream=None):
        check(lib().nexus_switch_key(self._h, ct.data_ptr(), ct.shape[1], target.data_ptr(), key.data_ptr(),
                                     _stream_ptr(stream)), "nexus_switch_key")

    def switch_key_batch(self, cts, targets, key, stream=None):
        """cts [B][2][limbs][N], targets [B][limbs][N]: every ciphertext in one pass."""
        check(lib().nexus_switch_key_batch(self._h, cts.data_ptr(), cts.shape[0], cts.shape[2], targets.data_ptr(),
                                           key.data_ptr(), _stream_ptr(stream)), "nexus_switch_key_batch")

    def relinearize(self, ct3, key, out2, stream=None):
        check(lib().nexus_relinearize(self._h, ct3.data_ptr(), ct3.shape[1], key.data_ptr(), out2.data_ptr(),
                                      _stream_ptr(stream)), "nexus_relinearize")

    def apply_galois(self, ct, elt, key, out, stream=None):
        check(lib().nexus_apply_galois(self._h, ct.data_ptr(), ct.shape[1], int(elt), key.data_ptr(),
                                       out.data_ptr(), _stream_ptr(stream)), "nexus_apply_galois")

    def autotune(self, limbs: int, batch: int, reps: int = 3) -> dict:
        """Choose the launch parameters by timing a batched key switch at this
        shape (nexus_autotune); returns the choice and its ms per call."""
        w, g, ms = C.c_int(), C.c_int(), C.c_double()
        check(lib().nexus_autotune(self._h, int(limbs), int(batch), int(reps), C.byref(w), C.byref(g), C.byref(ms)),
              "nexus_autotune")
        return {"ntt_prefetch_waves": w.value, "ks_inner_ctas_per_sm": g.value, "ntt_form": self.ntt_form(),
                "ms_per_call": ms.value}

    def set_tuning(self, ntt_prefetch_waves: int, ks_inner_ctas_per_sm: int) -> None:
        check(lib().nexus_set_tuning(self._h, int(ntt_prefetch_waves), int(ks_inner_ctas_per_sm)), "nexus_set_tuning")

    def tuning(self) -> dict:
        w, g = C.c_int(), C.c_int()
        check(lib().nexus_get_tuning(self._h, C.byref(w), C.byref(g)), "nexus_get_tuning")
        return {"ntt_prefetch_waves": w.value, "ks_inner_ctas_per_sm": g.value, "ntt_form": self.ntt_form()}

    def set_ntt_form(self, form: int) -> None:
        """0: forward NTT in two launches (default); 1: one launch of
        thread-block clusters holding each limb in distributed shared memory;
        2: two launches, the rows pass on rows of several limbs of one prime."""
        check(lib().nexus_set_ntt_form(self._h, int(form)), "nexus_set_ntt_form")

    def ntt_form(self) -> int:
        f = C.c_int()
        check(lib().nexus_get_ntt_form(self._h, C.byref(f)), "nexus_get_ntt_form")
        return f.value

    def galois_elt(self, step: int) -> int:
        e = C.c_uint32()
        check(lib().nexus_galois_elt_from_step(self.log_n, int(step), C.byref(e)), "galois_elt")
        return e.value

    def add(self, a, b, out, stream=None):
        check(lib().nexus_add(self._h, a.data_ptr(), b.data_ptr(), a.shape[0], a.shape[1], out.data_ptr(),
                              _stream_ptr(stream)), "nexus_add")

    def sub(self, a, b, out, stream=None):
        check(lib().nexus_sub(self._h, a.data_ptr(), b.data_ptr(), a.shape[0], a.shape[1], out.data_ptr(),
                              _stream_ptr(stream)), "nexus_sub")

    def negate(self, a, out, stream=None):
        check(lib().nexus_negate(self._h, a.data_ptr(), a.shape[0], a.shape[1], out.data_ptr(), _stream_ptr(stream)),
              "nexus_negate")

    def plain_op(self, ct, pt, op: int, out, stream=None):
        check(lib().nexus_plain_op(self._h, ct.data_ptr(), ct.shape[0], ct.shape[1], pt.data_ptr(), op,
                                   out.data_ptr(), _stream_ptr(stream)), "nexus_plain_op")

    # ---- encoding ----------------------------------------------------------
    def encode(self, values, scale: float, limbs: int, out, stream=None):
        v = np.asarray(values)
        re = np.ascontiguousarray(v.real, dtype=np.float64)
        im = np.ascontiguousarray(v.imag, dtype=np.float64) if np.iscomplexobj(v) else None
        check(lib().nexus_encode(self._h, re.ctypes.data, None if im is None else im.ctypes.data, re.size,
                                 float(scale), limbs, out.data_ptr(), _stream_ptr(stream)), "nexus_encode")

    def encode_scalar(self, value: float, scale: float, limbs: int) -> np.ndarray:
        out = np.zeros(limbs, dtype=np.uint64)
        check(lib().nexus_encode_scalar(self._h, float(value), float(scale), limbs,
                                        out.ctypes.data_as(C.POINTER(C.c_uint64))), "nexus_encode_scalar")
        return out

    def multiply_scalar(self, ct, per_limb, out, stream=None):
        pl = np.ascontiguousarray(per_limb, dtype=np.uint64)
        check(lib().nexus_multiply_scalar(self._h, ct.data_ptr(), ct.shape[0], ct.shape[1],
                                          pl.ctypes.data_as(C.POINTER(C.c_uint64)), out.data_ptr(),
                                          _stream_ptr(stream)), "nexus_multiply_scalar")

    def decode(self, pt, scale: float, nvals: int | None = None, sparse_slots: int = 0, stream=None):
        nvals = nvals or self.n // 2
        re = np.zeros(nvals)
        im = np.zeros(nvals)
        check(lib().nexus_decode(self._h, pt.data_ptr(), pt.shape[-2], float(scale), re.ctypes.data, im.ctypes.data,
                                 nvals, sparse_slots, _stream_ptr(stream)), "nexus_decode")
        return re + 1j * im

    # ---- keys, encryption, decryption ---------------------------------------
    def _empty(self, *shape):
        import torch
        return torch.empty(shape, dtype=torch.int64, device="cuda")

    def keygen_secret(self, seed: int, hamming_weight: int = 0, stream=None):
        sk = self._empty(len(self.moduli), self.n)
        check(lib().nexus_keygen_secret(self._h, int(seed), int(hamming_weight), sk.data_ptr(), _stream_ptr(stream)),
              "nexus_keygen_secret")
        return sk

    def keygen_relin(self, sk, seed: int, stream=None):
        k = len(self.moduli)
        key = self._empty(k - 1, 2, k, self.n)
        check(lib().nexus_keygen_relin(self._h, sk.data_ptr(), int(seed), key.data_ptr(), _stream_ptr(stream)),
              "nexus_keygen_relin")
        return key

    def keygen_galois(self, sk, elt: int, seed: int, stream=None):
        k = len(self.moduli)
        key = self._empty(k - 1, 2, k, self.n)
        check(lib().nexus_keygen_galois(self._h, sk.data_ptr(), int(elt), int(seed), key.data_ptr(),
                                        _stream_ptr(stream)), "nexus_keygen_galois")
        return key

    def encrypt_symmetric(self, sk, pt, limbs: int, seed: int, stream=None):
        ct = self._empty(2, limbs, self.n)
        check(lib().nexus_encrypt_symmetric(self._h, sk.data_ptr(), None if pt is None else pt.data_ptr(), limbs,
                                            int(seed), ct.data_ptr(), _stream_ptr(stream)), "nexus_encrypt_symmetric")
        return ct

    def decrypt(self, sk, ct, stream=None):
        size, limbs = ct.shape[0], ct.shape[1]
        pt = self._empty(limbs, self.n)
        check(lib().nexus_decrypt(self._h, sk.data_ptr(), ct.data_ptr(), size, limbs, pt.data_ptr(),
                                  _stream_ptr(stream)), "nexus_decrypt")
        return pt

    # ---- the same with SEAL's own randomness -----------------------------------
    # seed: an int (word 0 of SEAL's 8-word prng_seed_type, the rest zero) or 8
    # words; seeds of a key-switching key: one seed for all digits (what a
    # Blake2xbPRNGFactory with a default seed gives) or one per digit
    def _digit_seeds(self, seeds):
        k = len(self.moduli)
        a = np.asarray(seeds, dtype=np.uint64) if not isinstance(seeds, (int, np.integer)) else None
        if a is None or a.shape == (8,):
            one = seal_seed(seeds)
            return np.ascontiguousarray(np.tile(one, (k - 1, 1)))
        a = np.ascontiguousarray(a.reshape(-1, 8))
        if a.shape[0] != k - 1:
            raise ValueError(f"a key-switching key takes {k - 1} seeds, got {a.shape[0]}")
        return a

    def seal_keygen_secret(self, seed, hamming_weight: int = 0, stream=None):
        sk = self._empty(len(self.moduli), self.n)
        check(lib().nexus_seal_keygen_secret(self._h, _u64p(seal_seed(seed)), int(hamming_weight), sk.data_ptr(),
                                             _stream_ptr(stream)), "nexus_seal_keygen_secret")
        return sk

    def seal_keygen_public(self, sk, seed, stream=None):
        pk = self._empty(2, len(self.moduli), self.n)
        check(lib().nexus_seal_keygen_public(self._h, _u64p(seal_seed(seed)), sk.data_ptr(), pk.data_ptr(),
                                             _stream_ptr(stream)), "nexus_seal_keygen_public")
        return pk

    def seal_keygen_relin(self, sk, seeds, stream=None):
        k = len(self.moduli)
        key = self._empty(k - 1, 2, k, self.n)
        check(lib().nexus_seal_keygen_relin(self._h, _u64p(self._digit_seeds(seeds)), sk.data_ptr(), key.data_ptr(),
                                            _stream_ptr(stream)), "nexus_seal_keygen_relin")
        return key

    def seal_keygen_galois(self, sk, elt: int, seeds, stream=None):
        k = len(self.moduli)
        key = self._empty(k - 1, 2, k, self.n)
        check(lib().nexus_seal_keygen_galois(self._h, _u64p(self._digit_seeds(seeds)), sk.data_ptr(), int(elt),
                                             key.data_ptr(), _stream_ptr(stream)), "nexus_seal_keygen_galois")
        return key

    def seal_encrypt(self, pk, pt, limbs: int, seed, stream=None):
        ct = self._empty(2, limbs, self.n)
        check(lib().nexus_seal_encrypt(self._h, _u64p(seal_seed(seed)), pk.data_ptr(),
                                       None if pt is None else pt.data_ptr(), limbs, ct.data_ptr(),
                                       _stream_ptr(stream)), "nexus_seal_encrypt")
        return ct

    def seal_encrypt_symmetric(self, sk, pt, limbs: int, seed, stream=None):
        ct = self._empty(2, limbs, self.n)
        check(lib().nexus_seal_encrypt_symmetric(self._h, _u64p(seal_seed(seed)), sk.data_ptr(),
                                                 None if pt is None else pt.data_ptr(), limbs, ct.data_ptr(),
                                                 _stream_ptr(stream)), "nexus_seal_encrypt_symmetric")
        return ct

    def encode_coefficients(self, values, scale: float, limbs: int, out, stream=None):
        v = np.ascontiguousarray(values, dtype=np.float64)
        check(lib().nexus_encode_coefficients(self._h, v.ctypes.data, v.size, float(scale), limbs, out.data_ptr(),
                                              _stream_ptr(stream)), "nexus_encode_coefficients")

    # ---- measurement ---------------------------------------------------------
    def ntt_timing_begin(self):
        check(lib().nexus_ntt_timing_begin(self._h), "nexus_ntt_timing_begin")

    def ntt_timing_end(self):
        ms, calls, limbs = C.c_double(), C.c_uint64(), C.c_uint64()
        check(lib().nexus_ntt_timing_end(self._h, C.byref(ms), C.byref(calls), C.byref(limbs)), "nexus_ntt_timing_end")
        return ms.value, calls.value, limbs.value


def kernel_launches() -> int:
    return int(lib().nexus_kernel_launches())


def memory_info() -> dict:
    """Bytes of the engine's device memory pool (nexus_memory_info): live
    allocations now, their peak, what the pool holds, and what instantiated
    graphs hold for their allocations."""
    v = [C.c_uint64() for _ in range(4)]
    check(lib().nexus_memory_info(*[C.byref(x) for x in v]), "nexus_memory_info")
    return {"pool_used": v[0].value, "pool_used_high": v[1].value, "pool_reserved": v[2].value,
            "graph_reserved": v[3].value}


def memory_trim() -> None:
    """Return the engine pool's free blocks to the device (nexus_memory_trim)."""
    check(lib().nexus_memory_trim(), "nexus_memory_trim")


def butterfly_rate(mode: int, q: int, rounds: int = 512, blocks_per_sm: int = 3) -> float:
    """Butterflies per second of the NTT's own butterfly on this GPU (mode 0
    forward, 1 forward for primes below 2^52, 2 inverse): the compute ceiling
    of the transform (nexus_butterfly_rate)."""
    out = C.c_double()
    ms = C.c_double()
    check(lib().nexus_butterfly_rate(int(mode), C.c_uint64(int(q)), int(rounds), int(blocks_per_sm), C.byref(out),
                                     C.byref(ms)), "nexus_butterfly_rate")
    return out.value


TENSOR_BF16, TENSOR_E4M3 = 0, 1
TENSOR_M, TENSOR_N, TENSOR_ROW_BYTES = 128, 256, 128


def tensor_rate(kind: int, rounds: int = 20000) -> tuple[float, float]:
    """(FLOP/s, ms per launch) of hand-written tcgen05.mma on this GPU, one
    CTA per SM: kind 0 bf16 (kind::f16), 1 e4m3 (kind::f8f6f4)
    (nexus_tensor_rate)."""
    out = C.c_double()
    ms = C.c_double()
    check(lib().nexus_tensor_rate(int(kind), int(rounds), C.byref(out), C.byref(ms)), "nexus_tensor_rate")
    return out.value, ms.value


def tensor_tile(kind: int, a: np.ndarray, b: np.ndarray, rounds: int = 1) -> np.ndarray:
    """rounds * a . b^T through the tcgen05 kernel of tensor_rate on one CTA:
    a is 128 rows and b 256 rows of 128 operand bytes (uint16 bf16 bits or
    uint8 e4m3 bits); returns the 128 x 256 float32 accumulator
    (nexus_tensor_tile)."""
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.nbytes != TENSOR_M * TENSOR_ROW_BYTES or b.nbytes != TENSOR_N * TENSOR_ROW_BYTES:
        raise ValueError("a must hold 128 and b 256 rows of 128 bytes")
    d = np.empty((TENSOR_M, TENSOR_N), dtype=np.float32)
    check(lib().nexus_tensor_tile(int(kind), int(rounds), a.ctypes.data, b.ctypes.data, d.ctypes.data),
          "nexus_tensor_tile")
    return d
