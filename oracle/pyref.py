"""ctypes wrapper of oracle/_ref/libseal_shim.so (the real SEAL-4.1-bs) -- TEST INFRASTRUCTURE.

Available only where the NEXUS sources were present to build it; callers
check :func:`available` first.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libseal_shim.so"
_lib = None
u64p = C.POINTER(C.c_uint64)
f64p = C.POINTER(C.c_double)


def available() -> bool:
    if LIB_PATH.exists():
        return True
    try:
        from . import build_ref
        if build_ref.reference_available():
            build_ref.build()
            return LIB_PATH.exists()
    except Exception:
        return False
    return False


def lib():
    global _lib
    if _lib is None:
        l = C.CDLL(str(LIB_PATH))
        l.sr_last_error.restype = C.c_char_p
        l.sr_create.restype = C.c_void_p
        l.sr_create.argtypes = [C.c_int, u64p, C.c_int, C.c_uint64, C.c_int]
        l.sr_destroy.argtypes = [C.c_void_p]
        l.sr_keygen.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int]
        l.sr_export_secret.argtypes = [C.c_void_p, u64p]
        l.sr_export_relin.argtypes = [C.c_void_p, u64p]
        l.sr_export_galois.argtypes = [C.c_void_p, C.c_uint32, u64p]
        l.sr_galois_elt.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_uint32)]
        l.sr_ntt.argtypes = [C.c_int, C.c_uint64, u64p, C.c_size_t, C.c_int]
        l.sr_rescale.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, C.c_double, u64p, f64p]
        l.sr_multiply.argtypes = [C.c_void_p, u64p, u64p, C.c_int, u64p]
        l.sr_relinearize.argtypes = [C.c_void_p, u64p, C.c_int, u64p]
        l.sr_rotate.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p]
        l.sr_conjugate.argtypes = [C.c_void_p, u64p, C.c_int, u64p]
        l.sr_multiply_plain.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p, u64p]
        l.sr_encode.argtypes = [C.c_void_p, f64p, f64p, C.c_size_t, C.c_double, C.c_int, u64p]
        l.sr_encode_scalar.argtypes = [C.c_void_p, C.c_double, C.c_double, C.c_int, u64p]
        l.sr_decode.argtypes = [C.c_void_p, u64p, C.c_int, C.c_double, f64p, f64p, C.c_size_t]
        l.sr_encrypt.argtypes = [C.c_void_p, f64p, C.c_size_t, C.c_double, u64p]
        l.sr_decrypt.argtypes = [C.c_void_p, u64p, C.c_int, C.c_double, f64p, C.c_size_t]
        l.sr_nexus_op.argtypes = [C.c_void_p, C.c_int, u64p, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int,
                                  C.c_double, u64p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
        l.sr_fork_op.argtypes = [C.c_void_p, C.c_int, u64p, C.c_int, C.c_double, u64p, C.c_int, C.c_double,
                                 C.c_double, f64p, f64p, C.c_size_t, u64p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_double)]
        l.sr_galois_keys_from_elts.argtypes = [C.c_void_p, C.POINTER(C.c_uint32), C.c_int]
        l.sr_mm_compress.argtypes = [C.c_void_p, f64p, C.c_double, u64p, f64p]
        l.sr_mm_power_of_x.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p]
        l.sr_mm_expand.argtypes = [C.c_void_p, u64p, C.c_int, C.c_double, C.c_uint32, u64p]
        l.sr_parms_id.argtypes = [C.c_void_p, C.c_int, u64p]
        l.sr_ct_save.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, C.c_double, C.c_void_p, C.c_size_t,
                                 C.POINTER(C.c_size_t)]
        l.sr_ct_load.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, u64p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                 C.POINTER(C.c_double)]
        l.sr_create_seeded.restype = C.c_void_p
        l.sr_create_seeded.argtypes = [C.c_int, u64p, C.c_int, u64p, C.c_int]
        l.sr_create_seed_list.restype = C.c_void_p
        l.sr_create_seed_list.argtypes = [C.c_int, u64p, C.c_int, u64p, C.c_int, C.c_int]
        l.sr_export_public.argtypes = [C.c_void_p, u64p]
        l.sr_encrypt_ntt.argtypes = [C.c_void_p, u64p, C.c_int, C.c_double, C.c_int, u64p]
        l.sr_prng_bytes.argtypes = [u64p, C.c_uint64, C.c_size_t, C.c_void_p]
        _lib = l
    return _lib


def _p(a):
    assert a.flags.c_contiguous
    return a.ctypes.data_as(u64p if a.dtype == np.uint64 else f64p)


def _ck(rc):
    if rc != 0:
        raise RuntimeError(lib().sr_last_error().decode())


def ntt(log_n: int, q: int, a: np.ndarray, inverse=False) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64).copy()
    _ck(lib().sr_ntt(log_n, q, _p(a), a.size >> log_n, 1 if inverse else 0))
    return a


def prng_bytes(seed, offset: int, n: int) -> bytes:
    """Bytes [offset, offset + n) of SEAL's Blake2xbPRNG stream for an 8-word seed."""
    sd = np.ascontiguousarray(seed, dtype=np.uint64)
    out = (C.c_uint8 * max(1, n))()
    _ck(lib().sr_prng_bytes(_p(sd), offset, n, out))
    return bytes(out)[:n]


class SealRef:
    """SEAL CKKS context with seeded keys over explicit primes."""

    def __init__(self, log_n, moduli, seed=1, hamming_weight=0, steps=()):
        self.log_n, self.n = log_n, 1 << log_n
        self.moduli = [int(q) for q in moduli]
        self.k = len(self.moduli)
        arr = np.array(self.moduli, dtype=np.uint64)
        if isinstance(seed, (int, np.integer)):
            self._h = lib().sr_create(log_n, _p(arr), self.k, seed, hamming_weight)
        elif np.ndim(seed) == 2:   # one 8-word seed per create() call, in call order
            sd = np.ascontiguousarray(seed, dtype=np.uint64)
            self._h = lib().sr_create_seed_list(log_n, _p(arr), self.k, _p(sd), sd.shape[0], hamming_weight)
        else:   # the full 8-word seed of the Blake2xbPRNGFactory
            sd = np.ascontiguousarray(seed, dtype=np.uint64)
            assert sd.shape == (8,)
            self._h = lib().sr_create_seeded(log_n, _p(arr), self.k, _p(sd), hamming_weight)
        if not self._h:
            raise RuntimeError(lib().sr_last_error().decode())
        st = (C.c_int * max(1, len(steps)))(*steps)
        _ck(lib().sr_keygen(self._h, st, len(steps)))

    def __del__(self):
        if getattr(self, "_h", None):
            lib().sr_destroy(self._h)
            self._h = None

    def secret_key(self):
        out = np.zeros((self.k, self.n), np.uint64)
        _ck(lib().sr_export_secret(self._h, _p(out)))
        return out

    def public_key(self):
        out = np.zeros((2, self.k, self.n), np.uint64)
        _ck(lib().sr_export_public(self._h, _p(out)))
        return out

    def encrypt_ntt(self, pt, scale=2.0 ** 40, symmetric=False):
        """Encryptor::encrypt (public key) or encrypt_symmetric of an NTT-form plaintext [limbs][N]."""
        pt = np.ascontiguousarray(pt, dtype=np.uint64)
        out = np.zeros((2,) + pt.shape, np.uint64)
        _ck(lib().sr_encrypt_ntt(self._h, _p(pt), pt.shape[0], scale, 1 if symmetric else 0, _p(out)))
        return out

    def relin_key(self):
        out = np.zeros((self.k - 1, 2, self.k, self.n), np.uint64)
        _ck(lib().sr_export_relin(self._h, _p(out)))
        return out

    def galois_elt(self, step):
        e = C.c_uint32()
        _ck(lib().sr_galois_elt(self._h, step, C.byref(e)))
        return e.value

    def galois_key(self, elt):
        out = np.zeros((self.k - 1, 2, self.k, self.n), np.uint64)
        _ck(lib().sr_export_galois(self._h, elt, _p(out)))
        return out

    def rescale(self, ct, scale=2.0 ** 40):
        size, limbs, n = ct.shape
        out = np.zeros((size, limbs - 1, n), np.uint64)
        sc = C.c_double()
        _ck(lib().sr_rescale(self._h, _p(np.ascontiguousarray(ct)), size, limbs, scale, _p(out), C.byref(sc)))
        return out, sc.value

    def multiply(self, a, b):
        limbs = a.shape[1]
        out = np.zeros((3, limbs, self.n), np.uint64)
        _ck(lib().sr_multiply(self._h, _p(np.ascontiguousarray(a)), _p(np.ascontiguousarray(b)), limbs, _p(out)))
        return out

    def relinearize(self, ct3):
        limbs = ct3.shape[1]
        out = np.zeros((2, limbs, self.n), np.uint64)
        _ck(lib().sr_relinearize(self._h, _p(np.ascontiguousarray(ct3)), limbs, _p(out)))
        return out

    def rotate(self, ct, step):
        out = np.zeros_like(ct)
        _ck(lib().sr_rotate(self._h, _p(np.ascontiguousarray(ct)), ct.shape[1], step, _p(out)))
        return out

    def conjugate(self, ct):
        out = np.zeros_like(ct)
        _ck(lib().sr_conjugate(self._h, _p(np.ascontiguousarray(ct)), ct.shape[1], _p(out)))
        return out

    def multiply_plain(self, ct, pt):
        out = np.zeros_like(ct)
        _ck(lib().sr_multiply_plain(self._h, _p(np.ascontiguousarray(ct)), ct.shape[0], ct.shape[1],
                                    _p(np.ascontiguousarray(pt)), _p(out)))
        return out

    def encode(self, values, scale, limbs):
        v = np.asarray(values)
        re = np.ascontiguousarray(v.real, dtype=np.float64)
        im = np.ascontiguousarray(v.imag if np.iscomplexobj(v) else np.zeros_like(re), dtype=np.float64)
        out = np.zeros((limbs, self.n), np.uint64)
        _ck(lib().sr_encode(self._h, _p(re), _p(im), re.size, scale, limbs, _p(out)))
        return out

    def encode_scalar(self, value, scale, limbs):
        out = np.zeros((limbs, self.n), np.uint64)
        _ck(lib().sr_encode_scalar(self._h, float(value), scale, limbs, _p(out)))
        return out

    def decode(self, pt, scale, nvals=None):
        nvals = nvals or self.n // 2
        re = np.zeros(nvals)
        im = np.zeros(nvals)
        _ck(lib().sr_decode(self._h, _p(np.ascontiguousarray(pt)), pt.shape[0], scale, _p(re), _p(im), nvals))
        return re + 1j * im

    def encrypt(self, values, scale):
        v = np.ascontiguousarray(values, dtype=np.float64)
        out = np.zeros((2, self.k - 1, self.n), np.uint64)
        _ck(lib().sr_encrypt(self._h, _p(v), v.size, scale, _p(out)))
        return out

    def decrypt(self, ct, scale, nvals=None):
        nvals = nvals or self.n // 2
        out = np.zeros(nvals)
        _ck(lib().sr_decrypt(self._h, _p(np.ascontiguousarray(ct)), ct.shape[1], scale, _p(out), nvals))
        return out

    def parms_id(self, limbs):
        out = np.zeros(4, np.uint64)
        _ck(lib().sr_parms_id(self._h, limbs, _p(out)))
        return out

    def save(self, ct, scale) -> bytes:
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        n = C.c_size_t()
        _ck(lib().sr_ct_save(self._h, _p(ct), ct.shape[0], ct.shape[1], scale, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.uint8)
        _ck(lib().sr_ct_save(self._h, _p(ct), ct.shape[0], ct.shape[1], scale, out.ctypes.data, out.size,
                             C.byref(n)))
        return out.tobytes()

    def load(self, data: bytes):
        buf = np.frombuffer(data, dtype=np.uint8)
        size, limbs, scale = C.c_int(), C.c_int(), C.c_double()
        big = np.zeros(16 * self.k * self.n, np.uint64)
        _ck(lib().sr_ct_load(self._h, buf.ctypes.data, buf.size, _p(big), C.byref(size), C.byref(limbs),
                             C.byref(scale)))
        return big[:size.value * limbs.value * self.n].reshape(size.value, limbs.value, self.n), scale.value

    OPS = {"gelu": 0, "softmax": 1, "layer_norm": 2, "sgn_eval": 3, "exp": 4, "inverse": 5, "invert_sqrt": 6}

    def nexus_op(self, op, ct, scale, base_scale, a1=0, a2=0, f=0.0):
        """Run NEXUS's own operator (src/*.cpp compiled against this SEAL)."""
        out = np.zeros((2, self.k - 1, self.n), np.uint64)
        ol = C.c_int()
        osc = C.c_double()
        _ck(lib().sr_nexus_op(self._h, self.OPS[op], _p(np.ascontiguousarray(ct)), ct.shape[1], scale, base_scale,
                              a1, a2, f, _p(out), C.byref(ol), C.byref(osc)))
        return np.ascontiguousarray(out.reshape(-1)[: 2 * ol.value * self.n].reshape(2, ol.value, self.n)), osc.value

    def galois_keys_from_elts(self, elts):
        arr = (C.c_uint32 * len(elts))(*elts)
        _ck(lib().sr_galois_keys_from_elts(self._h, arr, len(elts)))

    def mm_compress(self, values, scale):
        v = np.ascontiguousarray(values, dtype=np.float64)
        out = np.zeros((2, self.k - 1, self.n), np.uint64)
        sc = C.c_double()
        _ck(lib().sr_mm_compress(self._h, _p(v), scale, _p(out), C.byref(sc)))
        return out, sc.value

    def mm_power_of_x(self, ct, index):
        out = np.zeros_like(ct)
        _ck(lib().sr_mm_power_of_x(self._h, _p(np.ascontiguousarray(ct)), ct.shape[1], index, _p(out)))
        return out

    def mm_expand(self, ct, scale, m):
        out = np.zeros((m, 2, ct.shape[1], self.n), np.uint64)
        _ck(lib().sr_mm_expand(self._h, _p(np.ascontiguousarray(ct)), ct.shape[1], scale, m, _p(out)))
        return out

    FORK = {"add_const": 0, "multiply_const": 1, "add_reduced_error": 2, "sub_reduced_error": 3,
            "multiply_reduced_error": 4, "multiply_vector_reduced_error": 5}

    def fork_op(self, op, a, sa, b=None, sb=0.0, value=0.0, vec=None):
        out = np.zeros((3, self.k - 1, self.n), np.uint64)
        osz, ol, osc = C.c_int(), C.c_int(), C.c_double()
        re = im = None
        nv = 0
        if vec is not None:
            vec = np.asarray(vec, dtype=np.complex128)
            re = np.ascontiguousarray(vec.real)
            im = np.ascontiguousarray(vec.imag)
            nv = vec.size
        _ck(lib().sr_fork_op(self._h, self.FORK[op], _p(np.ascontiguousarray(a)), a.shape[1], sa,
                             None if b is None else _p(np.ascontiguousarray(b)), 0 if b is None else b.shape[1], sb,
                             value, None if re is None else _p(re), None if im is None else _p(im), nv, _p(out),
                             C.byref(osz), C.byref(ol), C.byref(osc)))
        flat = out.reshape(-1)[: osz.value * ol.value * self.n]
        return np.ascontiguousarray(flat.reshape(osz.value, ol.value, self.n)), osc.value
