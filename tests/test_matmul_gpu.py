"""NEXUS MatMul (MMEvaluator) on the GPU engine against the oracle restatement
(oracle/nexus_l3.py, pinned to NEXUS on SEAL): multiply_power_of_x, the
expansion tree and the fused matrix_mul, word for word; plus the decrypted
product against FP64 X.W."""
import numpy as np
import pytest

from oracle import nexus_l3 as L
from oracle import pyoracle as po
from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu

LOG_N = 12
N = 1 << LOG_N
PT_SCALE = 2.0 ** 40
PACK_SCALE = 1e10  # enc_compress_ciphertext's fixed scale (src/matrix_mul.cpp:93)


@pytest.fixture(scope="module")
def env(cuda):
    import nexus_gb300 as ng
    from nexus_gb300.operators import Evaluator
    qs = ng.create_coeff_modulus(N, [60, 40, 60])
    ctx = ng.Context(LOG_N, qs)
    sk = ctx.keygen_secret(seed=31)
    rots = [(N + 2 ** i) // 2 ** i for i in range(LOG_N)]
    gks = {e: ctx.keygen_galois(sk, e, seed=100 + i) for i, e in enumerate(rots)}
    ev = Evaluator(ctx, PT_SCALE, None, gks)
    oc = po.OracleContext(LOG_N, qs)
    oev = L.Evaluator(oc, None, {e: to_host(k) for e, k in gks.items()})
    return ctx, sk, ev, L.MMEvaluator(L.CKKSEvaluator(oev, PT_SCALE))


def _compress(ctx, sk, values, seed):
    """enc_compress_ciphertext: encryption of zero + coefficient-packed values"""
    import torch
    from nexus_gb300.operators import Ciphertext
    ct = ctx.encrypt_symmetric(sk, None, 2, seed)
    pt = torch.empty((2, N), dtype=torch.int64, device="cuda")
    ctx.encode_coefficients(values, PACK_SCALE, 2, pt)
    c0 = ct[0:1].clone()
    ctx.plain_op(c0, pt, 1, ct[0:1])
    return Ciphertext.from_device(ctx, ct, PACK_SCALE), L.Ct(to_host(ct), PACK_SCALE)


def test_power_of_x(env):
    ctx, sk, ev, omm = env
    x, ox = _compress(ctx, sk, np.random.default_rng(0).uniform(-1, 1, N), 1)
    for idx in (0, 1, 7, N - 1, N, N + 5, 2 * N - 1):
        assert np.array_equal(ev.mm_power_of_x(x, idx).to_numpy(), omm.multiply_power_of_x(ox, idx).data), idx


@pytest.mark.parametrize("m", [4, 64, N])
def test_expand(env, m):
    ctx, sk, ev, omm = env
    x, ox = _compress(ctx, sk, np.random.default_rng(m).uniform(-1, 1, N), 2)
    got = to_host(ev.mm_expand(x, m))
    want = omm.expand_ciphertext(ox, m)
    for i in range(m):
        assert np.array_equal(got[i], want[i].data), i


def test_matrix_mul_two_packs(env):
    """6 x 1000 encrypted rows (spanning two compressed ciphertexts) times 1000 x 64 plaintext"""
    import torch
    ctx, sk, ev, omm = env
    rows, cols, outc = 6, 1000, 64
    rng = np.random.default_rng(5)
    X = rng.normal(0, 1, (rows, cols))
    W = rng.normal(0, 0.02, (cols, outc))
    flat = X.reshape(-1)
    packs = [_compress(ctx, sk, flat[i * N:(i + 1) * N], 10 + i) for i in range((flat.size + N - 1) // N)]
    pts = torch.empty((cols, 2, N), dtype=torch.int64, device="cuda")
    for k in range(cols):
        ctx.encode(W[k], PT_SCALE, 2, pts[k])
    res = ev.matrix_mul([p[0] for p in packs], pts, PT_SCALE, rows, cols, float(N))
    # oracle: full expansion of every pack, then the accumulation
    leaves = []
    for _, ox in packs:
        leaves += omm.expand_ciphertext(ox, N)
    opts = [L.Pt(PT_SCALE, data=to_host(pts[k])) for k in range(cols)]
    want = omm.accumulate(leaves, opts, rows, cols, float(N))
    for r in range(rows):
        assert res[r].scale == want[r].scale
        assert np.array_equal(res[r].to_numpy(), want[r].data), r
    # decrypted against FP64
    Y = X @ W
    for r in range(rows):
        dec = ctx.decode(ctx.decrypt(sk, res[r].to_device()), res[r].scale).real[:outc]
        assert np.max(np.abs(dec - Y[r])) < 1e-3
