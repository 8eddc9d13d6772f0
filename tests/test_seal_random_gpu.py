"""Key generation and encryption with SEAL's own randomness on the GPU
(nexus_seal_*): every word equal to SEAL-4.1-bs's for the same seeds --
against digests of the real SEAL (tests/golden/seal_keygen_kat.json, up to
the N=2^16 bootstrap chain) and against the oracle's full arrays."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle as po
from oracle import seal_random as sr

pytestmark = pytest.mark.gpu

KAT = json.loads((Path(__file__).parent / "golden" / "seal_keygen_kat.json").read_text())
CASES = {c["name"]: c for c in KAT["configs"]}


def _digest(t) -> str:
    h = hashlib.sha256()
    for part in t.reshape(t.shape[0], -1):    # keys are ~1 GB at N=2^16: one digit at a time
        h.update(part.cpu().numpy().view(np.uint64).astype("<u8").tobytes())
    return h.hexdigest()


def _np(t):
    return t.cpu().numpy().view(np.uint64)


def _pt(ctx, seed, log_n, moduli):
    import torch
    import nexus_gb300 as ng
    a = ng.seal_sample_poly(seed, ng.SEAL_UNIFORM, log_n, moduli)
    return torch.from_numpy(a.view(np.int64)).cuda()


@pytest.mark.parametrize("name", list(CASES))
def test_engine_matches_seal_digests(name):
    import torch
    import nexus_gb300 as ng
    c = CASES[name]
    qs = [int(q) for q in c["moduli"]]
    ctx = ng.Context(c["log_n"], qs)
    seed = np.array(c["seed"], dtype=np.uint64)
    if "error" in c:
        with pytest.raises(ng.NexusError, match=c["error"]):
            ctx.seal_keygen_secret(seed, c["hamming_weight"])
        return
    sk = ctx.seal_keygen_secret(seed, c["hamming_weight"])
    pk = ctx.seal_keygen_public(sk, seed)
    got = {"secret_key": _digest(sk), "public_key": _digest(pk)}
    if c["relin"]:
        rk = ctx.seal_keygen_relin(sk, seed)
        got["relin_key"] = _digest(rk)
        del rk
    for st in c["steps"]:
        gk = ctx.seal_keygen_galois(sk, ctx.galois_elt(st), seed)
        got[f"galois_key_step_{st}"] = _digest(gk)
        del gk
    for limbs in c["enc_limbs"]:
        pt = _pt(ctx, c["pt_seed"], c["log_n"], qs[:limbs])
        got[f"encrypt_l{limbs}"] = _digest(ctx.seal_encrypt(pk, pt, limbs, seed))
        got[f"encrypt_symmetric_l{limbs}"] = _digest(ctx.seal_encrypt_symmetric(sk, pt, limbs, seed))
    torch.cuda.synchronize()
    assert got == c["sha256"]


@pytest.mark.parametrize("hw", [0, 64])
def test_engine_matches_oracle_with_a_seed_per_digit(hw):
    # the default factory draws a fresh seed per create(): every digit of a
    # key-switching key and every encryption has its own stream
    import nexus_gb300 as ng
    log_n, n = 12, 1 << 12
    qs = po.create_coeff_modulus(n, [50, 40, 40, 50])
    k = len(qs)
    ctx = ng.Context(log_n, qs)
    kg = sr.SealKeygen(po.OracleContext(log_n, qs))
    seeds = [np.arange(8 * j + 1, 8 * j + 9, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15) for j in range(8)]
    sk = ctx.seal_keygen_secret(seeds[0], hw)
    osk = kg.secret_key(seeds[0], hw)
    assert np.array_equal(_np(sk), osk)
    pk = ctx.seal_keygen_public(sk, seeds[1])
    opk = kg.public_key(seeds[1], osk)
    assert np.array_equal(_np(pk), opk)
    dseeds = seeds[2:2 + k - 1]
    assert np.array_equal(_np(ctx.seal_keygen_relin(sk, np.stack(dseeds))), kg.relin_key(dseeds, osk))
    elt = ctx.galois_elt(-5)
    assert np.array_equal(_np(ctx.seal_keygen_galois(sk, elt, np.stack(dseeds))), kg.galois_key(dseeds, osk, elt))
    for limbs in (3, 2, 1):
        pt = _pt(ctx, 100 + limbs, log_n, qs[:limbs])
        opt = _np(pt)
        assert np.array_equal(_np(ctx.seal_encrypt(pk, pt, limbs, seeds[6])), kg.encrypt(seeds[6], opk, opt, limbs))
        assert np.array_equal(_np(ctx.seal_encrypt_symmetric(sk, pt, limbs, seeds[7])),
                              kg.encrypt_symmetric(seeds[7], osk, opt, limbs))
        assert np.array_equal(_np(ctx.seal_encrypt(pk, None, limbs, seeds[6])), kg.encrypt(seeds[6], opk, None, limbs))


def test_seal_encryptions_decrypt_to_the_message():
    import torch
    import nexus_gb300 as ng
    log_n, n = 13, 1 << 13
    qs = po.create_coeff_modulus(n, [60, 40, 40, 60])
    ctx = ng.Context(log_n, qs)
    sk = ctx.seal_keygen_secret(11, 0)
    pk = ctx.seal_keygen_public(sk, 12)
    vals = np.random.default_rng(3).uniform(-1, 1, n // 2)
    scale = 2.0 ** 40
    for limbs in (3, 1):
        pt = torch.empty((limbs, n), dtype=torch.int64, device="cuda")
        ctx.encode(vals, scale, limbs, pt)
        for ct in (ctx.seal_encrypt(pk, pt, limbs, 13), ctx.seal_encrypt_symmetric(sk, pt, limbs, 14)):
            dec = ctx.decode(ctx.decrypt(sk, ct), scale).real
            assert np.max(np.abs(dec - vals)) < 1e-6
