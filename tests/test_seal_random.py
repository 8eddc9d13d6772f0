"""SEAL's seeded randomness without a GPU: the oracle's BLAKE2b / BLAKE2Xb
stream, samplers, key generation and encryption against digests of the real
SEAL-4.1-bs (tests/golden/seal_keygen_kat.json) and, where the reference is
built here, against SEAL itself; the engine's host-side stream and samplers
(nexus_seal_prng_bytes, nexus_seal_sample_poly) against the oracle."""
import ctypes as C
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import seal_random as sr

KAT = json.loads((Path(__file__).parent / "golden" / "seal_keygen_kat.json").read_text())
CASES = {c["name"]: c for c in KAT["configs"]}


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def test_oracle_blake2b_is_rfc7693_blake2b():
    # the written-out compression against CPython's BLAKE2b: a plain hash and
    # the keyed XOF root (fanout 1, depth 1, XOF length in the node offset)
    for msg in (b"", b"abc", bytes(range(100))):
        block = np.frombuffer(msg.ljust(128, b"\0"), dtype="<u8")
        h = sr._compress(sr._param(64, 0, 1, 1, 0, 0, 0, 0, 0), [int(w) for w in block], len(msg), True)
        assert np.array(h, dtype="<u8").tobytes() == hashlib.blake2b(msg).digest()
    for seed, counter in ((sr.seed_words(1), 0), (np.arange(5, 13, dtype=np.uint64), 12345)):
        root = np.array(sr.blake2xb_root(seed, counter), dtype="<u8").tobytes()
        ref = hashlib.blake2b(counter.to_bytes(8, "little"), key=seed.astype("<u8").tobytes(), digest_size=64,
                              node_offset=sr.REFILL << 32).digest()
        assert root == ref


@pytest.mark.parametrize("case", KAT["streams"])
def test_oracle_stream_is_seal_stream(case):
    assert sr.Stream(case["seed"], case["offset"]).bytes(case["n"]).hex() == case["hex"]


def test_engine_stream_matches_oracle_and_seal():
    import nexus_gb300 as ng
    for case in KAT["streams"]:
        assert ng.seal_prng_bytes(case["seed"], case["offset"], case["n"]).hex() == case["hex"]
    seed = np.arange(21, 29, dtype=np.uint64) * np.uint64(0x100000001B3)
    for off, n in ((0, 3 * 4096 + 5), (4095, 9), (70001, 50000)):
        assert ng.seal_prng_bytes(seed, off, n) == sr.Stream(seed, off).bytes(n)


@pytest.mark.parametrize("seed", [1, 5, 6, 16, list(range(3, 11))])
def test_engine_samplers_match_oracle(seed):
    import nexus_gb300 as ng
    log_n, n = 10, 1 << 10
    qs = po.create_coeff_modulus(n, [40, 30, 40])
    for off in (0, 64, 4093):
        assert np.array_equal(ng.seal_sample_poly(seed, ng.SEAL_TERNARY, log_n, qs, offset=off),
                              sr.small_to_rns(sr.sample_ternary(sr.Stream(seed, off), n), qs))
        assert np.array_equal(ng.seal_sample_poly(seed, ng.SEAL_CBD, log_n, qs, offset=off),
                              sr.small_to_rns(sr.sample_cbd(sr.Stream(seed, off), n), qs))
        assert np.array_equal(ng.seal_sample_poly(seed, ng.SEAL_SPARSE_TERNARY, log_n, qs, 192, offset=off),
                              sr.sample_sparse_ternary(sr.Stream(seed, off), n, qs, 192))
        assert np.array_equal(ng.seal_sample_poly(seed, ng.SEAL_UNIFORM, log_n, qs, offset=off),
                              sr.sample_uniform(sr.Stream(seed, off), n, qs))


def test_sparse_sampler_position_n_writes_the_next_rows():
    # seed 6 draws position N once with a negative sign: coefficient 0 of
    # rows 1 and 2 take the residues of -1 modulo the row before
    n = 1 << 10
    qs = po.create_coeff_modulus(n, [40, 30, 40])
    v = sr.sample_sparse_ternary(sr.Stream(6), n, qs, 192)
    assert v[1, 0] == qs[0] - 1 and v[2, 0] == qs[1] - 1
    assert np.count_nonzero(v[0]) == 191


def _oracle_outputs(c):
    qs = [int(q) for q in c["moduli"]]
    ctx = po.OracleContext(c["log_n"], qs)
    kg = sr.SealKeygen(ctx)
    seed = np.array(c["seed"], dtype=np.uint64)
    out = {}
    sk = kg.secret_key(seed, c["hamming_weight"])
    pk = kg.public_key(seed, sk)
    out["secret_key"], out["public_key"] = sk, pk
    seeds = [seed] * (len(qs) - 1)
    if c["relin"]:
        out["relin_key"] = kg.relin_key(seeds, sk)
    for st in c["steps"]:
        out[f"galois_key_step_{st}"] = kg.galois_key(seeds, sk, po.galois_elt_from_step(c["log_n"], st))
    for limbs in c["enc_limbs"]:
        pt = sr.sample_uniform(sr.Stream(c["pt_seed"]), 1 << c["log_n"], qs[:limbs])
        out[f"encrypt_l{limbs}"] = kg.encrypt(seed, pk, pt, limbs)
        out[f"encrypt_symmetric_l{limbs}"] = kg.encrypt_symmetric(seed, sk, pt, limbs)
    return out


@pytest.mark.parametrize("name", ["n4096_dense", "n4096_sparse_reduced"])
def test_oracle_keygen_and_encryption_match_seal_digests(name):
    c = CASES[name]
    got = {k: digest(v) for k, v in _oracle_outputs(c).items()}
    assert got == c["sha256"]


def test_oracle_rejects_the_key_seal_rejects():
    c = CASES["n4096_sparse_invalid"]
    assert c["error"] == "secret key is not valid for encryption parameters"
    kg = sr.SealKeygen(po.OracleContext(c["log_n"], [int(q) for q in c["moduli"]]))
    with pytest.raises(ValueError, match=c["error"]):
        kg.secret_key(np.array(c["seed"], dtype=np.uint64), c["hamming_weight"])


def test_oracle_matches_live_seal():
    from oracle import pyref
    if not pyref.available():
        pytest.skip("SEAL reference build unavailable")
    log_n, n = 11, 1 << 11
    qs = po.create_coeff_modulus(n, [45, 36, 36, 45])
    for seed, hw in ((sr.seed_words(31), 0), (np.arange(40, 48, dtype=np.uint64), 100)):
        ref = pyref.SealRef(log_n, qs, seed=seed, hamming_weight=hw, steps=[2])
        kg = sr.SealKeygen(po.OracleContext(log_n, qs))
        sk = kg.secret_key(seed, hw)
        assert np.array_equal(sk, ref.secret_key())
        pk = kg.public_key(seed, sk)
        assert np.array_equal(pk, ref.public_key())
        seeds = [seed] * 3
        assert np.array_equal(kg.relin_key(seeds, sk), ref.relin_key())
        e = ref.galois_elt(2)
        assert np.array_equal(kg.galois_key(seeds, sk, e), ref.galois_key(e))
        for limbs in (3, 1):
            pt = sr.sample_uniform(sr.Stream(99), n, qs[:limbs])
            assert np.array_equal(kg.encrypt(seed, pk, pt, limbs), ref.encrypt_ntt(pt))
            assert np.array_equal(kg.encrypt_symmetric(seed, sk, pt, limbs), ref.encrypt_ntt(pt, symmetric=True))


def test_oracle_matches_live_seal_with_a_seed_per_call():
    # a factory handing every create() its own seed: SEAL draws the secret
    # key, the public key, each relinearisation digit, each Galois digit and
    # each encryption from separate streams, in that order
    from oracle import pyref
    if not pyref.available():
        pytest.skip("SEAL reference build unavailable")
    log_n, n = 11, 1 << 11
    qs = po.create_coeff_modulus(n, [45, 36, 36, 45])
    k = len(qs)
    calls = 2 + 2 * (k - 1) + 2
    seeds = (np.arange(calls * 8, dtype=np.uint64).reshape(calls, 8) + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
    for hw in (0, 64):
        ref = pyref.SealRef(log_n, qs, seed=seeds, hamming_weight=hw, steps=[3])
        kg = sr.SealKeygen(po.OracleContext(log_n, qs))
        sk = kg.secret_key(seeds[0], hw)
        assert np.array_equal(sk, ref.secret_key())
        pk = kg.public_key(seeds[1], sk)
        assert np.array_equal(pk, ref.public_key())
        assert np.array_equal(kg.relin_key(list(seeds[2:k + 1]), sk), ref.relin_key())
        e = ref.galois_elt(3)
        assert np.array_equal(kg.galois_key(list(seeds[k + 1:2 * k]), sk, e), ref.galois_key(e))
        pt = sr.sample_uniform(sr.Stream(5), n, qs[:2])
        assert np.array_equal(kg.encrypt(seeds[2 * k], pk, pt, 2), ref.encrypt_ntt(pt))
        assert np.array_equal(kg.encrypt_symmetric(seeds[2 * k + 1], sk, pt, 2), ref.encrypt_ntt(pt, symmetric=True))


def test_seal_entry_points_reject_bad_arguments_without_gpu():
    from nexus_gb300 import _lib
    lib = _lib.lib()
    seed = np.zeros(8, dtype=np.uint64)
    sp = seed.ctypes.data_as(C.POINTER(C.c_uint64))
    q = np.array([97], dtype=np.uint64)
    qp = q.ctypes.data_as(C.POINTER(C.c_uint64))
    out = np.zeros(8, dtype=np.uint64)
    op = out.ctypes.data_as(C.POINTER(C.c_uint64))
    cases = [
        ("nexus_seal_prng_bytes", lambda: lib.nexus_seal_prng_bytes(None, 0, 4, None), b"null"),
        ("nexus_seal_sample_poly", lambda: lib.nexus_seal_sample_poly(sp, 0, 9, 3, qp, 1, 0, op), b"kind"),
        ("nexus_seal_sample_poly", lambda: lib.nexus_seal_sample_poly(sp, 0, 1, 3, qp, 1, 0, op), b"hamming"),
        ("nexus_seal_keygen_secret", lambda: lib.nexus_seal_keygen_secret(None, sp, 0, None, None), b"null"),
        ("nexus_seal_keygen_public", lambda: lib.nexus_seal_keygen_public(None, sp, None, None, None), b"null"),
        ("nexus_seal_keygen_relin", lambda: lib.nexus_seal_keygen_relin(None, sp, None, None, None), b"null"),
        ("nexus_seal_keygen_galois", lambda: lib.nexus_seal_keygen_galois(None, sp, None, 3, None, None), b"null"),
        ("nexus_seal_encrypt", lambda: lib.nexus_seal_encrypt(None, sp, None, None, 1, None, None), b"null"),
        ("nexus_seal_encrypt_symmetric", lambda: lib.nexus_seal_encrypt_symmetric(None, sp, None, None, 1, None, None),
         b"null"),
    ]
    for name, call, word in cases:
        assert call() != 0, name
        msg = lib.nexus_last_error()
        assert msg.startswith(name.encode()) and word in msg, (name, msg)
