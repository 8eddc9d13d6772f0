"""SEAL byte format of CKKS ciphertexts (Ciphertext::save / load with
compr_mode none): the engine's host serializer against bytes SEAL itself
wrote (committed fixture, tests/golden/make_seal_bytes.py) and, where the
SEAL build exists, live round trips through SEAL."""
from pathlib import Path

import numpy as np
import pytest

from nexus_gb300.operators import seal_load, seal_save
from nexus_gb300._lib import NexusError

FIX = np.load(Path(__file__).parent / "golden" / "seal_ciphertext_bytes.npz")


@pytest.mark.parametrize("name", ["a", "b3"])
def test_save_matches_seal_bytes(name):
    want = FIX[f"{name}_bytes"].tobytes()
    got = seal_save(FIX[f"{name}_words"], float(FIX[f"{name}_scale"]), FIX[f"{name}_pid"])
    assert got == want


@pytest.mark.parametrize("name", ["a", "b3"])
def test_load_seal_bytes(name):
    words, scale, pid, ntt = seal_load(FIX[f"{name}_bytes"].tobytes())
    assert np.array_equal(words, FIX[f"{name}_words"])
    assert scale == float(FIX[f"{name}_scale"])
    assert np.array_equal(pid, FIX[f"{name}_pid"])
    assert ntt


def test_load_rejects_malformed_bytes():
    good = bytearray(FIX["a_bytes"].tobytes())
    bad_magic = bytearray(good)
    bad_magic[0] ^= 0xFF
    with pytest.raises(NexusError, match="SEALHeader is invalid"):
        seal_load(bytes(bad_magic))
    zlib = bytearray(good)
    zlib[5] = 1
    with pytest.raises(NexusError, match="compression"):
        seal_load(bytes(zlib))
    with pytest.raises(NexusError):
        seal_load(bytes(good[:-8]))
    with pytest.raises(NexusError):
        seal_load(bytes(good[:20]))


def test_round_trip_through_seal():
    from oracle import pyoracle as po
    from oracle import pyref as pr
    if not pr.available():
        pytest.skip("SEAL reference build unavailable")
    log_n, n = 13, 1 << 13
    qs = po.create_coeff_modulus(n, [58, 40, 40, 58])
    s = pr.SealRef(log_n, qs, seed=3)
    ct = s.encrypt(np.random.default_rng(1).uniform(-1, 1, n // 2), 2.0 ** 40)
    for limbs in (3, 2, 1):
        c = np.ascontiguousarray(ct[:, :limbs, :])
        ours = seal_save(c, 2.0 ** 40, s.parms_id(limbs))
        assert ours == s.save(c, 2.0 ** 40)
        words, scale = s.load(ours)
        assert np.array_equal(words, c) and scale == 2.0 ** 40


@pytest.mark.gpu
def test_engine_ciphertext_round_trip(cuda):
    import nexus_gb300 as ng
    from nexus_gb300.operators import Ciphertext
    from oracle import pyoracle as po
    n = 1 << 12
    qs = po.create_coeff_modulus(n, [50, 40, 50])
    ctx = ng.Context(12, qs)
    ct, pid = Ciphertext.load_seal(ctx, FIX["a_bytes"].tobytes())
    assert np.array_equal(ct.to_numpy(), FIX["a_words"]) and ct.scale == float(FIX["a_scale"])
    assert ct.save_seal(pid) == FIX["a_bytes"].tobytes()
