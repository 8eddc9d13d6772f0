"""SEAL-4.1-bs's seeded randomness, key generation and encryption restated on
the CPU -- TEST INFRASTRUCTURE (the oracle; never shipped or timed as the
product).

Stream.  Blake2xbPRNG (native/src/seal/randomgen.cpp:197-207, randomgen.h:504-530)
refills a 4096-byte buffer with BLAKE2Xb(key = the 64-byte seed, message =
the 8-byte little-endian refill counter, 4096 bytes of output) and hands the
bytes out in order (UniformRandomGenerator::generate, randomgen.cpp:174-190).
BLAKE2b is restated from RFC 7693 in plain Python and BLAKE2Xb from the
BLAKE2X specification (Aumasson et al. 2016): the root is keyed BLAKE2b-512
with fanout 1, depth 1 and the XOF length in the upper half of the 64-bit
node-offset field; output block i is unkeyed BLAKE2b-512 of the root with
fanout 0, depth 0, leaf length 64, inner length 64 and node offset i (same
XOF length).  Python's hashlib cannot express depth 0, so the compression
function is written out.  The NEXUS tree vendors the BLAKE2 reference
package for this (thirdparty/SEAL-4.1-bs/native/src/seal/util/blake2xb.c).

Samplers (native/src/seal/util/rlwe.cpp): sample_poly_ternary :21-37,
sample_poly_sparse_ternary :39-69 (the NEXUS fork), sample_poly_cbd :99-135
(SEAL's default noise sampler), sample_poly_uniform :137-165.  Ternary draws
go through std::uniform_int_distribution<uint64_t> over 32-bit draws, which
libstdc++ (GCC 11+) computes with Lemire's nearly divisionless method
(ACM TOMACS 29(1), 2019), restated in :func:`uniform_int`.

Flows: KeyGenerator::generate_sk / generate_pk / generate_one_kswitch_key
(native/src/seal/keygenerator.cpp:56-93, 95-122, 303-336), encrypt_zero_symmetric
(util/rlwe.cpp:311-441), encrypt_zero_asymmetric (util/rlwe.cpp:224-309) and
Encryptor::encrypt_zero_internal / encrypt_internal (encryptor.cpp:88-237).

Pinned against the real SEAL (oracle/_ref, tests/test_seal_random.py) and
against digests of SEAL's outputs (tests/golden/seal_keygen_kat.json).
"""
from __future__ import annotations

import numpy as np

from .pyoracle import OracleContext, galois_table_ntt

REFILL = 4096
SEED_WORDS = 8


def seed_words(seed) -> np.ndarray:
    """An int (SEAL's prng_seed_type with word 0 set, the rest zero) or 8 words."""
    if isinstance(seed, (int, np.integer)):
        w = np.zeros(SEED_WORDS, dtype=np.uint64)
        w[0] = int(seed)
        return w
    w = np.asarray(seed, dtype=np.uint64)
    assert w.shape == (SEED_WORDS,)
    return w


_M64 = (1 << 64) - 1
# RFC 7693 section 2.6 (initial value) and 2.7 (message schedule)
_IV = (0x6a09e667f3bcc908, 0xbb67ae8584caa73b, 0x3c6ef372fe94f82b, 0xa54ff53a5f1d36f1,
       0x510e527fade682d1, 0x9b05688c2b3e6c1f, 0x1f83d9abfb41bd6b, 0x5be0cd19137e2179)
_SIGMA = ((0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15), (14, 10, 4, 8, 9, 15, 13, 6, 1, 12, 0, 2, 11, 7, 5, 3),
          (11, 8, 12, 0, 5, 2, 15, 13, 10, 14, 3, 6, 7, 1, 9, 4), (7, 9, 3, 1, 13, 12, 11, 14, 2, 6, 5, 10, 4, 0, 15, 8),
          (9, 0, 5, 7, 2, 4, 10, 15, 14, 1, 11, 12, 6, 8, 3, 13), (2, 12, 6, 10, 0, 11, 8, 3, 4, 13, 7, 5, 15, 14, 1, 9),
          (12, 5, 1, 15, 14, 13, 4, 10, 0, 7, 6, 3, 9, 2, 8, 11), (13, 11, 7, 14, 12, 1, 3, 9, 5, 0, 15, 4, 8, 6, 2, 10),
          (6, 15, 14, 9, 11, 3, 0, 8, 12, 2, 13, 7, 1, 4, 10, 5), (10, 2, 8, 4, 7, 6, 1, 5, 15, 11, 9, 14, 3, 12, 13, 0))
_G_LANES = ((0, 4, 8, 12), (1, 5, 9, 13), (2, 6, 10, 14), (3, 7, 11, 15),
            (0, 5, 10, 15), (1, 6, 11, 12), (2, 7, 8, 13), (3, 4, 9, 14))


def _compress(h, m, t, last):
    """RFC 7693 section 3.2: BLAKE2b compression of the 16-word block m."""
    v = list(h) + list(_IV)
    v[12] ^= t
    if last:
        v[14] ^= _M64
    for r in range(12):
        s = _SIGMA[r % 10]
        for g, (a, b, c, d) in enumerate(_G_LANES):
            x, y = m[s[2 * g]], m[s[2 * g + 1]]
            v[a] = (v[a] + v[b] + x) & _M64
            w = v[d] ^ v[a]
            v[d] = (w >> 32) | ((w << 32) & _M64)
            v[c] = (v[c] + v[d]) & _M64
            w = v[b] ^ v[c]
            v[b] = (w >> 24) | ((w << 40) & _M64)
            v[a] = (v[a] + v[b] + y) & _M64
            w = v[d] ^ v[a]
            v[d] = (w >> 16) | ((w << 48) & _M64)
            v[c] = (v[c] + v[d]) & _M64
            w = v[b] ^ v[c]
            v[b] = (w >> 63) | ((w << 1) & _M64)
    return [h[i] ^ v[i] ^ v[i + 8] for i in range(8)]


def _param(digest, key, fanout, depth, leaf, node_offset, xof_len, node_depth, inner):
    """BLAKE2b initial state for a BLAKE2X parameter block (first three words)."""
    h = list(_IV)
    h[0] ^= digest | (key << 8) | (fanout << 16) | (depth << 24) | (leaf << 32)
    h[1] ^= node_offset | (xof_len << 32)
    h[2] ^= node_depth | (inner << 8)
    return h


def blake2xb_root(seed, counter: int):
    """Keyed BLAKE2b-512 of the counter with the XOF length in the parameter block."""
    key = [int(w) for w in seed_words(seed)]
    h = _compress(_param(64, 64, 1, 1, 0, 0, REFILL, 0, 0), key + [0] * 8, 128, False)
    return _compress(h, [int(counter)] + [0] * 15, 136, True)


_CACHE: dict = {}


def blake2xb_refill(seed, counter: int) -> bytes:
    tag = (seed_words(seed).tobytes(), int(counter))
    hit = _CACHE.get(tag)
    if hit is not None:
        return hit
    root = blake2xb_root(seed, counter) + [0] * 8
    out = b"".join(np.array(_compress(_param(64, 0, 0, 0, 64, i, REFILL, 0, 64), root, 64, True),
                            dtype="<u8").tobytes() for i in range(REFILL // 64))
    if len(_CACHE) > 4096:
        _CACHE.clear()
    _CACHE[tag] = out
    return out


class Stream:
    """The byte stream of one Blake2xbPRNG."""

    def __init__(self, seed, offset: int = 0):
        self.seed = seed_words(seed)
        self.pos = int(offset)
        self._block = -1
        self._buf = b""

    def bytes(self, n: int) -> bytes:
        out = bytearray()
        while n:
            b, off = divmod(self.pos, REFILL)
            if b != self._block:
                self._buf, self._block = blake2xb_refill(self.seed, b), b
            take = min(n, REFILL - off)
            out += self._buf[off:off + take]
            self.pos += take
            n -= take
        return bytes(out)

    def u32_array(self, n: int) -> np.ndarray:
        return np.frombuffer(self.bytes(4 * n), dtype="<u4").astype(np.uint64)

    def u64(self) -> int:
        return int.from_bytes(self.bytes(8), "little")


def uniform_int(stream: Stream, lo: int, hi: int) -> int:
    r = hi - lo + 1
    product = int(stream.u32_array(1)[0]) * r
    low = product & 0xFFFFFFFF
    if low < r:
        threshold = ((1 << 32) - r) % r
        while low < threshold:
            product = int(stream.u32_array(1)[0]) * r
            low = product & 0xFFFFFFFF
    return lo + (product >> 32)


def sample_ternary(stream: Stream, n: int) -> np.ndarray:
    return np.array([uniform_int(stream, 0, 2) - 1 for _ in range(n)], dtype=np.int64)


_POP = np.array([bin(i).count("1") for i in range(256)], dtype=np.int64)


def sample_cbd(stream: Stream, n: int) -> np.ndarray:
    x = np.frombuffer(stream.bytes(6 * n), dtype=np.uint8).reshape(n, 6).copy()
    x[:, 2] &= 0x1F
    x[:, 5] &= 0x1F
    p = _POP[x]
    return p[:, 0] + p[:, 1] + p[:, 2] - p[:, 3] - p[:, 4] - p[:, 5]


def sample_sparse_ternary(stream: Stream, n: int, moduli, hw: int) -> np.ndarray:
    """[k][n] residues; position n (the fork's inclusive range) writes
    coefficient 0 of rows 1..k-1 with the previous row's residue and one word
    past the array, which is dropped."""
    k = len(moduli)
    a = [0] * (k * n + 1)
    weight = 0
    while weight < hw:
        index = uniform_int(stream, 0, n)
        if a[index] != 0:
            continue
        neg = uniform_int(stream, 0, 1) == 0
        for i in range(k):
            a[index + i * n] = int(moduli[i]) - 1 if neg else 1
        weight += 1
    return np.array(a[:k * n], dtype=np.uint64).reshape(k, n)


def uniform_bound(q: int) -> int:
    m = (1 << 64) - 1
    return m - (m % q) - 1


def sample_uniform(stream: Stream, n: int, moduli) -> np.ndarray:
    k = len(moduli)
    raw = np.frombuffer(stream.bytes(8 * k * n), dtype="<u8").astype(np.uint64).reshape(k, n).copy()
    for j, q in enumerate(moduli):
        bound = uniform_bound(int(q))
        for i in np.nonzero(raw[j] >= np.uint64(bound))[0]:
            v = int(raw[j, i])
            while v >= bound:
                v = stream.u64()
            raw[j, i] = v
        raw[j] %= np.uint64(q)
    return raw


def small_to_rns(v: np.ndarray, moduli) -> np.ndarray:
    q = np.array([int(x) for x in moduli], dtype=object).reshape(-1, 1)
    return (np.asarray(v, dtype=object).reshape(1, -1) % q).astype(np.uint64)


class SealKeygen:
    """The key generation and encryption flows over an OracleContext whose
    primes are the key level (data primes, then the special prime)."""

    def __init__(self, ctx: OracleContext):
        self.ctx = ctx
        self.n = ctx.n
        self.k = ctx.k
        self.q = ctx.moduli

    def _ntt(self, a, limbs):
        return self.ctx.ntt(a, 0, limbs)

    def _neg(self, a):
        return self.ctx.sub(np.zeros_like(a), a)

    def secret_key(self, seed, hamming_weight=0) -> np.ndarray:
        st = Stream(seed)
        if hamming_weight:
            v = sample_sparse_ternary(st, self.n, self.q, hamming_weight)
            # ntt_negacyclic_harvey (util/ntt.cpp:408-440) reduces inputs below
            # 4q canonically; a larger residue left by the position-n write
            # makes SEAL's key fail is_valid_for
            for r in range(1, self.k):
                x = int(v[r, 0])
                if x >= self.q[r]:
                    if x >= 4 * self.q[r]:
                        raise ValueError("secret key is not valid for encryption parameters")
                    v[r, 0] = x % self.q[r]
        else:
            v = small_to_rns(sample_ternary(st, self.n), self.q)
        return self._ntt(v, self.k)

    def encrypt_zero_symmetric(self, seed, sk, limbs) -> np.ndarray:
        boot = Stream(seed)
        pub = np.frombuffer(boot.bytes(64), dtype="<u8").astype(np.uint64)
        c1 = sample_uniform(Stream(pub), self.n, self.q[:limbs])
        e = self._ntt(small_to_rns(sample_cbd(boot, self.n), self.q[:limbs]), limbs)
        as_ = self.ctx.multiply_plain(c1[None], np.ascontiguousarray(sk[:limbs]))[0]
        c0 = self._neg(self.ctx.add(as_[None], e[None]))[0]
        return np.stack([c0, c1])

    def public_key(self, seed, sk) -> np.ndarray:
        return self.encrypt_zero_symmetric(seed, sk, self.k)

    def kswitch_key(self, seeds, sk, new_key) -> np.ndarray:
        p = self.q[-1]
        out = []
        for j in range(self.k - 1):
            ct = self.encrypt_zero_symmetric(seeds[j], sk, self.k)
            f = p % self.q[j]
            term = (new_key[j].astype(object) * f % self.q[j]).astype(np.uint64)
            ct[0, j] = ((ct[0, j].astype(object) + term.astype(object)) % self.q[j]).astype(np.uint64)
            out.append(ct)
        return np.stack(out)

    def relin_key(self, seeds, sk) -> np.ndarray:
        s2 = self.ctx.multiply_plain(sk[None], sk)[0]
        return self.kswitch_key(seeds, sk, s2)

    def galois_key(self, seeds, sk, elt) -> np.ndarray:
        tab = galois_table_ntt(self.ctx.log_n, elt).astype(np.int64)
        return self.kswitch_key(seeds, sk, np.ascontiguousarray(sk[:, tab]))

    def encrypt_symmetric(self, seed, sk, pt, limbs) -> np.ndarray:
        ct = self.encrypt_zero_symmetric(seed, sk, limbs)
        if pt is not None:
            ct[0] = self.ctx.add(ct[:1], np.asarray(pt, dtype=np.uint64)[None])[0]
        return ct

    def encrypt(self, seed, pk, pt, limbs) -> np.ndarray:
        """Encryptor::encrypt with the public key pk [2][k][n]."""
        up = limbs + 1 if limbs < self.k else limbs
        st = Stream(seed)
        u = self._ntt(small_to_rns(sample_ternary(st, self.n), self.q[:up]), up)
        e = [self._ntt(small_to_rns(sample_cbd(st, self.n), self.q[:up]), up) for _ in range(2)]
        c = np.stack([self.ctx.add(self.ctx.multiply_plain(np.ascontiguousarray(pk[j, :up])[None], u), e[j][None])[0]
                      for j in range(2)])
        if up > limbs:
            c = self.ctx.rescale(c)
        if pt is not None:
            c[0] = self.ctx.add(c[:1], np.asarray(pt, dtype=np.uint64)[None])[0]
        return c
