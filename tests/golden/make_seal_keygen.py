"""Generate tests/golden/seal_keygen_kat.json with the real SEAL-4.1-bs library:
SHA-256 digests of the secret key, public key, relinearization key, Galois
keys and public-key / secret-key encryptions that SEAL makes from a seeded
Blake2xbPRNGFactory (every create() call gets the same 8-word seed), plus
the first bytes of two raw Blake2xbPRNG streams.

Plaintexts are the uniform residues that SEAL's sample_poly_uniform draws
from the stream of `pt_seed` (a stand-in for any NTT-form plaintext).  A
digest is taken over the little-endian bytes of the uint64 array in SEAL's
layout ([limbs][N], [2][limbs][N], [n_moduli-1][2][n_moduli][N]).

Run where the NEXUS sources are available (the SEAL build in oracle/_ref
needs them):  python tests/golden/make_seal_keygen.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pyoracle as po  # noqa: E402
from oracle import pyref as pr  # noqa: E402
from oracle import seal_random as sr  # noqa: E402

BOOT_BITS = [51] + [46] * 16 + [51] * 14 + [51]

CONFIGS = [
    # small chain, dense ternary secret, 8-word seed; keys and encryptions
    dict(name="n4096_dense", log_n=12, bits=[50, 40, 40, 50], seed=[int(0x9E3779B97F4A7C15 * i % 2 ** 64)
                                                                    for i in range(1, 9)],
         hamming_weight=0, steps=[1, -3], pt_seed=77, enc_limbs=[3, 1], relin=True),
    # sparse secret whose position-N draw leaves a residue below 4q (reduced)
    dict(name="n4096_sparse_reduced", log_n=12, bits=[30, 29, 40], seed=[75] + [0] * 7, hamming_weight=192,
         steps=[], pt_seed=78, enc_limbs=[2], relin=True),
    # the same draw with a residue above 4q: SEAL rejects the key
    dict(name="n4096_sparse_invalid", log_n=12, bits=[40, 30, 40], seed=[75] + [0] * 7, hamming_weight=192,
         steps=[], pt_seed=0, enc_limbs=[], relin=False),
    # the bootstrap chain at N=2^16 with NEXUS's h=192 sparse secret
    dict(name="n65536_boot_sparse", log_n=16, bits=BOOT_BITS, seed=[2024] + [0] * 7, hamming_weight=192,
         steps=[1], pt_seed=79, enc_limbs=[31, 1], relin=True),
]

STREAMS = [dict(seed=[1] + [0] * 7, offset=0, n=256), dict(seed=list(range(100, 108)), offset=4000, n=256)]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def plaintext(pt_seed: int, log_n: int, moduli) -> np.ndarray:
    return sr.sample_uniform(sr.Stream(pt_seed), 1 << log_n, moduli)


def main():
    assert pr.available(), "SEAL reference build unavailable"
    out = {"configs": [], "streams": []}
    for c in CONFIGS:
        n = 1 << c["log_n"]
        qs = po.create_coeff_modulus(n, c["bits"])
        rec = dict(c, moduli=[str(q) for q in qs], sha256={})
        seed = np.array(c["seed"], dtype=np.uint64)
        try:
            ref = pr.SealRef(c["log_n"], qs, seed=seed, hamming_weight=c["hamming_weight"], steps=c["steps"])
        except RuntimeError as e:
            rec["error"] = str(e)
            out["configs"].append(rec)
            print(c["name"], "error:", e, flush=True)
            continue
        d = rec["sha256"]
        d["secret_key"] = digest(ref.secret_key())
        d["public_key"] = digest(ref.public_key())
        if c["relin"]:
            d["relin_key"] = digest(ref.relin_key())
        for st in c["steps"]:
            d[f"galois_key_step_{st}"] = digest(ref.galois_key(ref.galois_elt(st)))
        for limbs in c["enc_limbs"]:
            pt = plaintext(c["pt_seed"], c["log_n"], qs[:limbs])
            d[f"encrypt_l{limbs}"] = digest(ref.encrypt_ntt(pt, symmetric=False))
            d[f"encrypt_symmetric_l{limbs}"] = digest(ref.encrypt_ntt(pt, symmetric=True))
        out["configs"].append(rec)
        print(c["name"], "done", flush=True)
    for s in STREAMS:
        b = pr.prng_bytes(np.array(s["seed"], dtype=np.uint64), s["offset"], s["n"])
        out["streams"].append(dict(s, hex=b.hex()))
    (Path(__file__).parent / "seal_keygen_kat.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
