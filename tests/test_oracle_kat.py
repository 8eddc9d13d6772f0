"""Pin the CPU oracle to SEAL's own known-answer vectors (tests/golden/seal_kat.json)."""
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po

KAT = json.loads((Path(__file__).parent / "golden" / "seal_kat.json").read_text())


def test_ntt_tables_roots():
    k = KAT["ntt_tables"]
    q = k["modulus"]
    for logn, key in ((1, "root_powers_logn1"), (2, "root_powers_logn2")):
        c = po.OracleContext(logn, [q])
        rp, irp = c.root_powers(0)
        assert [int(x) for x in rp] == k[key]
        if logn == 1:
            # inverse table slot 1 holds the inverse of root power 1 (ntt.cpp:62-64)
            assert int(irp[1]) == po.lib().or_invmod(int(rp[1]), q)


def test_negacyclic_ntt_kat():
    k = KAT["negacyclic_ntt"]
    c = po.OracleContext(k["log_n"], [k["modulus"]])
    for inp, exp in k["cases"]:
        out = c.ntt(np.array(inp, dtype=np.uint64), 0, 1)
        assert [int(x) for x in out] == exp
        back = c.ntt(out, 0, 1, inverse=True)
        assert [int(x) for x in back] == inp


def test_inverse_ntt_round_trip_logn3():
    q = KAT["ntt_tables"]["modulus"]
    c = po.OracleContext(3, [q])
    rng = np.random.default_rng(7)
    for _ in range(100):
        x = rng.integers(0, q, 8, dtype=np.uint64)
        assert np.array_equal(c.ntt(c.ntt(x, 0, 1), 0, 1, inverse=True), x)
    assert np.array_equal(c.ntt(np.zeros(8, np.uint64), 0, 1, inverse=True), np.zeros(8, np.uint64))


def test_divide_and_round_q_last_kat():
    k = KAT["divide_and_round_q_last"]
    q0, q1 = k["moduli"]
    c = po.OracleContext(k["log_n"], k["moduli"])
    for case in k["cases"]:
        x = np.array(case["in"], dtype=np.uint64).reshape(1, 2, 2)
        x = c.ntt(x, 0, 2)
        out = c.rescale(x)  # [1][1][2]
        res = c.ntt(out, 0, 1, inverse=True).reshape(-1)
        for got, want in zip(res, case["expect"]):
            assert (q0 + want - int(got)) % q0 <= 1


def test_galois_ntt_kat():
    k = KAT["galois_ntt"]
    tab = po.galois_table_ntt(k["log_n"], k["galois_elt"])
    inp = np.array(k["input"])
    assert [int(inp[t]) for t in tab] == k["output"]


def test_coeff_modulus_shape():
    # CoeffModulus::Create: primes are 1 mod 2N, of the requested size, distinct
    n = 1 << 14
    bits = [60] + [40] * 7 + [60]
    qs = po.create_coeff_modulus(n, bits)
    assert len(set(qs)) == len(qs)
    for q, b in zip(qs, bits):
        assert q.bit_length() == b and q % (2 * n) == 1 and po.lib().or_is_prime(q)


def test_primitive_root_is_minimal():
    q = po.create_coeff_modulus(1 << 10, [30])[0]
    deg = 1 << 11
    r = po.minimal_primitive_root(deg, q)
    assert pow(r, deg // 2, q) == q - 1
    # brute force over all odd powers
    allr = {pow(r, e, q) for e in range(1, deg, 2)}
    assert r == min(allr)
