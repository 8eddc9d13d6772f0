"""NEXUS operators on the GPU engine against the oracle restatement
(oracle/nexus_l3.py, itself pinned to NEXUS-on-SEAL), word for word, plus the
decrypted accuracy against FP64."""
import math

import numpy as np
import pytest

from oracle import nexus_l3 as L
from oracle import pyoracle as po
from tests.util import to_host

pytestmark = pytest.mark.gpu

LOG_N = 12
N = 1 << LOG_N
SCALE = 2.0 ** 40
STEPS = [-128] + [2 ** i for i in range(7)]


@pytest.fixture(scope="module")
def env(cuda):
    import nexus_gb300 as ng
    from nexus_gb300.operators import Evaluator
    qs = ng.create_coeff_modulus(N, [58] + [40] * 24 + [58])
    ctx = ng.Context(LOG_N, qs)
    sk = ctx.keygen_secret(seed=21)
    rk = ctx.keygen_relin(sk, seed=22)
    gks = {ctx.galois_elt(st): ctx.keygen_galois(sk, ctx.galois_elt(st), seed=23 + i) for i, st in enumerate(STEPS)}
    ev = Evaluator(ctx, SCALE, rk, gks)
    oc = po.OracleContext(LOG_N, qs)
    oev = L.Evaluator(oc, to_host(rk), {e: to_host(k) for e, k in gks.items()})
    return ctx, sk, ev, L.CKKSEvaluator(oev, SCALE)


def _encrypt(ctx, sk, values, seed):
    import torch
    from nexus_gb300.operators import Ciphertext
    pt = torch.empty((len(ctx.moduli) - 1, N), dtype=torch.int64, device="cuda")
    ctx.encode(values, SCALE, pt.shape[0], pt)
    ct = ctx.encrypt_symmetric(sk, pt, pt.shape[0], seed)
    return Ciphertext.from_device(ctx, ct, SCALE), L.Ct(to_host(ct), SCALE)


def _decrypt(ctx, sk, ct):
    t = ct.to_device()
    return ctx.decode(ctx.decrypt(sk, t), ct.scale).real


def _same(eng, orc):
    assert eng.scale == orc.scale
    assert np.array_equal(eng.to_numpy(), orc.data)


def gelu_ref(x):
    return 0.5 * x * (1 + np.tanh(math.sqrt(2 / math.pi) * (x + 0.044715 * x ** 3)))


def test_gelu(env):
    ctx, sk, ev, ock = env
    v = np.random.default_rng(0).uniform(-5, 5, N // 2)
    x, ox = _encrypt(ctx, sk, v, 1)
    out = ev.gelu(x)
    _same(out, L.gelu(ock, ox))
    err = np.abs(_decrypt(ctx, sk, out) - gelu_ref(v))
    assert err.max() < 0.05 and err.mean() < 5e-3


def test_softmax(env):
    ctx, sk, ev, ock = env
    v = np.random.default_rng(1).uniform(-5, 0, N // 2)
    x, ox = _encrypt(ctx, sk, v, 2)
    out = ev.softmax(x, 128)
    _same(out, L.softmax(ock, ox, 128))


def test_layer_norm(env):
    ctx, sk, ev, ock = env
    v = np.random.default_rng(2).uniform(-1, 1, N // 2)
    x, ox = _encrypt(ctx, sk, v, 3)
    out = ev.layer_norm(x, 128)
    _same(out, L.layer_norm(ock, ox, 128))


@pytest.mark.parametrize("op", ["sgn", "exp", "inverse", "invert_sqrt"])
def test_primitives(env, op):
    ctx, sk, ev, ock = env
    lo, hi = {"sgn": (-1, 1), "exp": (-4, 0), "inverse": (0.1, 1.9), "invert_sqrt": (0.01, 5)}[op]
    v = np.random.default_rng(3).uniform(lo, hi, N // 2)
    x, ox = _encrypt(ctx, sk, v, 4)
    if op == "sgn":
        out, want, ref = ev.sgn_eval(x, 2, 2, 0.5), ock.sgn_eval(ox, 2, 2, 0.5), None
    elif op == "exp":
        out, want, ref = ev.exp(x), ock.exp(ox), (1 + v / 128) ** 128
    elif op == "inverse":
        out, want, ref = ev.inverse(x, 4), ock.inverse(ox, 4), None
    else:
        out, want, ref = ev.invert_sqrt(x, 5, 2), ock.invert_sqrt(ox, 5, 2), None
    _same(out, want)
    if ref is not None:
        assert np.max(np.abs(_decrypt(ctx, sk, out) - ref)) < 1e-3


def test_errors_match_seal_conditions(env):
    """level exhaustion raises SEAL's error text instead of faulting"""
    import torch
    from nexus_gb300 import NexusError
    from nexus_gb300.operators import Ciphertext
    ctx, sk, ev, ock = env
    pt = torch.empty((2, N), dtype=torch.int64, device="cuda")
    ctx.encode(np.ones(4), SCALE, 2, pt)
    ct = ctx.encrypt_symmetric(sk, pt, 2, 9)
    x = Ciphertext.from_device(ctx, ct, SCALE)
    with pytest.raises(NexusError, match="scale out of bounds|end of modulus|level too low"):
        ev.gelu(x)


def test_lockstep_operators_equal_single(env):
    """gelu / softmax / layer_norm / sgn / exp / inverse / invert_sqrt on three
    ciphertexts in lockstep give each ciphertext the single form's words."""
    from nexus_gb300.operators import OP_EXP, OP_INVERSE, OP_INVERT_SQRT, OP_SGN_EVAL
    ctx, sk, ev, ock = env
    rng = np.random.default_rng(40)

    def fresh(lo, hi):
        vals = [rng.uniform(lo, hi, N // 2) for _ in range(3)]
        return lambda: [_encrypt(ctx, sk, v, 100 + i)[0] for i, v in enumerate(vals)]

    cases = [
        (fresh(-5, 5), lambda xs: ev.gelu_batch(xs), lambda x: ev.gelu(x)),
        (fresh(-5, 0), lambda xs: ev.softmax_batch(xs, 128), lambda x: ev.softmax(x, 128)),
        (fresh(-1, 1), lambda xs: ev.layer_norm_batch(xs, 128), lambda x: ev.layer_norm(x, 128)),
        (fresh(-1, 1), lambda xs: ev.ckks_op_batch(OP_SGN_EVAL, xs, 2, 2, 0.5), lambda x: ev.sgn_eval(x, 2, 2, 0.5)),
        (fresh(-1, 0), lambda xs: ev.ckks_op_batch(OP_EXP, xs), lambda x: ev.exp(x)),
        (fresh(0.5, 1.5), lambda xs: ev.ckks_op_batch(OP_INVERSE, xs, 4), lambda x: ev.inverse(x, 4)),
        (fresh(1, 100), lambda xs: ev.ckks_op_batch(OP_INVERT_SQRT, xs, 5, 2), lambda x: ev.invert_sqrt(x, 5, 2)),
    ]
    for make, batched, single in cases:
        got = batched(make())
        for g, x in zip(got, make()):
            want = single(x)
            assert g.scale == want.scale
            assert np.array_equal(g.to_numpy(), want.to_numpy())


def test_inputs_are_validated(env):
    """An empty ciphertext or one of another context is an error, not a kernel
    launch on missing or mis-sized data."""
    import nexus_gb300 as ng
    from nexus_gb300 import NexusError
    from nexus_gb300.operators import Ciphertext
    ctx, sk, ev, ock = env
    with pytest.raises(NexusError, match="empty"):
        ev.gelu(Ciphertext(ctx))
    other = ng.Context(LOG_N, ng.create_coeff_modulus(N, [50, 40, 50]))
    foreign = Ciphertext.from_numpy(other, np.zeros((2, 2, N), dtype=np.uint64), SCALE)
    with pytest.raises(NexusError, match="another context"):
        ev.exp(foreign)
    with pytest.raises(NexusError, match="another context"):
        ev.gelu_batch([foreign])


def test_gelu_on_the_short_chain_fails_like_seal(cuda):
    """GELU needs 18 rescales; on 60 + 7 x 40 + 60 SEAL stops with "scale out
    of bounds" (NEXUS on SEAL, N=2^14), and so does the engine."""
    import torch
    import nexus_gb300 as ng
    from nexus_gb300 import NexusError
    from nexus_gb300.operators import Ciphertext, Evaluator
    n = 1 << 14
    qs = ng.create_coeff_modulus(n, [60] + [40] * 7 + [60])
    ctx = ng.Context(14, qs)
    sk = ctx.keygen_secret(seed=5)
    ev = Evaluator(ctx, SCALE, ctx.keygen_relin(sk, seed=6))
    top = len(qs) - 1
    pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
    ctx.encode(np.random.default_rng(0).uniform(-5, 5, n // 2), SCALE, top, pt)
    x = Ciphertext.from_device(ctx, ctx.encrypt_symmetric(sk, pt, top, 7), SCALE)
    with pytest.raises(NexusError, match="scale out of bounds|end of modulus switching chain|level too low"):
        ev.gelu(x)
