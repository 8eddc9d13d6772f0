"""Keygen / encrypt / decrypt round trips on the GPU with the engine's own keys."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.util import to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup(cuda):
    from nexus_gb300 import Context, create_coeff_modulus
    log_n = 14
    qs = create_coeff_modulus(1 << log_n, [60, 40, 40, 40, 60])
    ctx = Context(log_n, qs)
    sk = ctx.keygen_secret(seed=7)
    return ctx, sk, qs


def test_secret_key_is_ternary(setup):
    ctx, sk, qs = setup
    oc = po.OracleContext(ctx.log_n, qs)
    coeffs = oc.ntt(to_host(sk), 0, len(qs), inverse=True)
    q = np.array(qs, dtype=np.uint64).reshape(-1, 1)
    signed = np.where(coeffs > q // np.uint64(2), -(q - coeffs).astype(np.int64), coeffs.astype(np.int64))
    assert set(np.unique(signed)) <= {-1, 0, 1}
    assert np.all(signed == signed[0])  # same small integer in every prime


def test_sparse_secret_weight(cuda):
    from nexus_gb300 import Context, create_coeff_modulus
    qs = create_coeff_modulus(1 << 13, [50, 40, 50])
    ctx = Context(13, qs)
    sk = ctx.keygen_secret(seed=3, hamming_weight=192)
    coeffs = po.OracleContext(13, qs).ntt(to_host(sk), 0, 3, inverse=True)
    assert int(np.count_nonzero(coeffs[0])) == 192


def test_encrypt_decrypt_round_trip(setup):
    import torch
    ctx, sk, qs = setup
    vals = np.random.default_rng(0).uniform(-1, 1, ctx.n // 2)
    pt = torch.empty((4, ctx.n), dtype=torch.int64, device="cuda")
    ctx.encode(vals, 2.0 ** 40, 4, pt)
    ct = ctx.encrypt_symmetric(sk, pt, 4, seed=11)
    dec = ctx.decode(ctx.decrypt(sk, ct), 2.0 ** 40).real
    assert np.max(np.abs(dec - vals)) < 1e-7


def test_relin_and_rotation_keys_work(setup):
    import torch
    ctx, sk, qs = setup
    rng = np.random.default_rng(1)
    a, b = rng.uniform(-1, 1, ctx.n // 2), rng.uniform(-1, 1, ctx.n // 2)
    scale = 2.0 ** 40
    pa = torch.empty((4, ctx.n), dtype=torch.int64, device="cuda")
    pb = torch.empty_like(pa)
    ctx.encode(a, scale, 4, pa)
    ctx.encode(b, scale, 4, pb)
    ca, cb = ctx.encrypt_symmetric(sk, pa, 4, 1), ctx.encrypt_symmetric(sk, pb, 4, 2)
    m3 = torch.empty((3, 4, ctx.n), dtype=torch.int64, device="cuda")
    ctx.multiply(ca, cb, m3)
    rk = ctx.keygen_relin(sk, seed=5)
    r = torch.empty_like(ca)
    ctx.relinearize(m3, rk, r)
    out = torch.empty((2, 3, ctx.n), dtype=torch.int64, device="cuda")
    ctx.rescale(r, out)
    dec = ctx.decode(ctx.decrypt(sk, out), scale * scale / qs[3]).real
    assert np.max(np.abs(dec - a * b)) < 1e-6
    # size-3 decryption equals relinearized decryption
    d3 = ctx.decode(ctx.decrypt(sk, m3), scale * scale).real
    assert np.max(np.abs(d3 - a * b)) < 1e-6
    for step in (1, 5, -3):
        elt = ctx.galois_elt(step)
        gk = ctx.keygen_galois(sk, elt, seed=9)
        rot = torch.empty_like(ca)
        ctx.apply_galois(ca, elt, gk, rot)
        dec = ctx.decode(ctx.decrypt(sk, rot), scale).real
        # key-switch noise with a 60-bit digit; SEAL shows ~1.1e-6 at these parameters
        assert np.max(np.abs(dec - np.roll(a, -step))) < 1e-5, step
    # conjugation of a real vector leaves it unchanged
    gk = ctx.keygen_galois(sk, ctx.galois_elt(0), seed=10)
    conj = torch.empty_like(ca)
    ctx.apply_galois(ca, ctx.galois_elt(0), gk, conj)
    assert np.max(np.abs(ctx.decode(ctx.decrypt(sk, conj), scale).real - a)) < 1e-5
