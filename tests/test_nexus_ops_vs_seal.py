"""NEXUS operators: the oracle restatement (oracle/nexus_l3.py) against NEXUS's
own src/*.cpp compiled against the real SEAL-4.1-bs, on SEAL's keys and
ciphertexts.  Word-for-word equality of the output ciphertext and its scale.
Skipped where the SEAL/NEXUS reference build is unavailable."""
import numpy as np
import pytest

from oracle import nexus_l3 as L
from oracle import pyoracle as po
from oracle import pyref as pr

pytestmark = pytest.mark.skipif(not pr.available(), reason="SEAL reference build unavailable")

LOG_N = 13
N = 1 << LOG_N
SCALE = 2.0 ** 40
STEPS = [-128, 128] + [2 ** i for i in range(7)] + [-(2 ** i) for i in range(7)]


@pytest.fixture(scope="module")
def env():
    qs = po.create_coeff_modulus(N, [58] + [40] * 24 + [58])
    s = pr.SealRef(LOG_N, qs, seed=5, steps=STEPS)
    oc = po.OracleContext(LOG_N, qs)
    gk = {s.galois_elt(st): s.galois_key(s.galois_elt(st)) for st in STEPS}
    ev = L.Evaluator(oc, s.relin_key(), gk)
    return s, L.CKKSEvaluator(ev, SCALE)


def _check(got, want):
    data, scale = want
    assert got.scale == scale
    assert np.array_equal(got.data, data)


def test_gelu(env):
    s, ck = env
    ct = s.encrypt(np.random.default_rng(0).uniform(-5, 5, N // 2), SCALE)
    _check(L.gelu(ck, L.Ct(ct, SCALE)), s.nexus_op("gelu", ct, SCALE, SCALE))


def test_softmax(env):
    s, ck = env
    ct = s.encrypt(np.random.default_rng(1).uniform(-5, 0, N // 2), SCALE)
    _check(L.softmax(ck, L.Ct(ct, SCALE), 128), s.nexus_op("softmax", ct, SCALE, SCALE, a1=128))


def test_layer_norm(env):
    s, ck = env
    ct = s.encrypt(np.random.default_rng(2).uniform(-1, 1, N // 2), SCALE)
    _check(L.layer_norm(ck, L.Ct(ct, SCALE), 128), s.nexus_op("layer_norm", ct, SCALE, SCALE, a1=128))


@pytest.mark.parametrize("op,args", [("sgn_eval", (2, 2, 0.5)), ("sgn_eval", (1, 3, 1.0)), ("exp", ()),
                                     ("inverse", (4,)), ("invert_sqrt", (5, 2)), ("invert_sqrt", (4, 1))])
def test_primitives(env, op, args):
    s, ck = env
    lo, hi = {"sgn_eval": (-1, 1), "exp": (-4, 0), "inverse": (0.1, 1.9), "invert_sqrt": (0.01, 5)}[op]
    ct = s.encrypt(np.random.default_rng(3).uniform(lo, hi, N // 2), SCALE)
    x = L.Ct(ct, SCALE)
    if op == "sgn_eval":
        got = ck.sgn_eval(x, *args)
        want = s.nexus_op(op, ct, SCALE, SCALE, a1=args[0], a2=args[1], f=args[2])
    elif op == "exp":
        got, want = ck.exp(x), s.nexus_op(op, ct, SCALE, SCALE)
    elif op == "inverse":
        got, want = ck.inverse(x, *args), s.nexus_op(op, ct, SCALE, SCALE, a1=args[0])
    else:
        got, want = ck.invert_sqrt(x, *args), s.nexus_op(op, ct, SCALE, SCALE, a1=args[0], a2=args[1])
    _check(got, want)


def test_naf_and_multi_rotation(env):
    """rotate by a step without its own key: SEAL's NAF decomposition"""
    s, ck = env
    ct = s.encrypt(np.random.default_rng(4).uniform(-1, 1, N // 2), SCALE)
    for step in (3, 7, 100, -5):
        assert np.array_equal(ck.ev.rotate(L.Ct(ct, SCALE), step).data, s.rotate(ct, step))
    assert L.naf(7) == [-1, 8] and L.naf(-6) == [2, -8]


@pytest.fixture(scope="module")
def mm_env():
    log_n, n = 13, 1 << 13
    qs = po.create_coeff_modulus(n, [60, 40, 60])
    s = pr.SealRef(log_n, qs, seed=9)
    rots = [(n + 2 ** i) // 2 ** i for i in range(log_n)]
    s.galois_keys_from_elts(rots)
    oc = po.OracleContext(log_n, qs)
    ev = L.Evaluator(oc, s.relin_key(), {e: s.galois_key(e) for e in rots})
    return s, L.MMEvaluator(L.CKKSEvaluator(ev, SCALE)), n


def test_matmul_power_of_x(mm_env):
    s, mm, n = mm_env
    ct, sc = s.mm_compress(np.random.default_rng(0).uniform(-1, 1, n), SCALE)
    for idx in (0, 1, 5, n - 1, n, n + 3, 2 * n - 1):
        assert np.array_equal(s.mm_power_of_x(ct, idx), mm.multiply_power_of_x(L.Ct(ct, sc), idx).data)


@pytest.mark.parametrize("m", [2, 16, 64])
def test_matmul_expand(mm_env, m):
    s, mm, n = mm_env
    ct, sc = s.mm_compress(np.random.default_rng(m).uniform(-1, 1, n), SCALE)
    want = s.mm_expand(ct, sc, m)
    got = mm.expand_ciphertext(L.Ct(ct, sc), m)
    assert len(got) == m
    for i in range(m):
        assert np.array_equal(want[i], got[i].data), i


@pytest.mark.parametrize("la,lb", [(5, 5), (3, 6), (6, 3)])
def test_fork_reduced_error_ops(env, la, lb):
    """add/sub/multiply_reduced_error, add_const, multiply_const and
    multiply_vector_reduced_error of the bootstrapping SEAL"""
    s, ck = env
    ev = ck.ev
    rng = np.random.default_rng(la * 10 + lb)
    ct_a = s.encrypt(rng.uniform(-1, 1, N // 2), SCALE)
    ct_b = s.encrypt(rng.uniform(-1, 1, N // 2), SCALE)
    a = L.Ct(np.ascontiguousarray(ct_a[:, :la]), SCALE * 1.0003)
    b = L.Ct(np.ascontiguousarray(ct_b[:, :lb]), SCALE * 0.9991)
    for op, fn in (("add_reduced_error", ev.add_reduced_error), ("sub_reduced_error", ev.sub_reduced_error),
                   ("multiply_reduced_error", ev.multiply_reduced_error)):
        want, wsc = s.fork_op(op, a.data, a.scale, b.data, b.scale)
        got = fn(a, b)
        assert got.scale == wsc and np.array_equal(got.data, want), op
    for op, fn, v in (("add_const", ev.add_const, 0.37), ("multiply_const", ev.multiply_const, -1.7)):
        want, wsc = s.fork_op(op, a.data, a.scale, value=v)
        got = fn(a, v)
        assert got.scale == wsc and np.array_equal(got.data, want), op
    vec = rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2)
    want, wsc = s.fork_op("multiply_vector_reduced_error", a.data, a.scale, vec=vec)
    got = ev.multiply_vector_reduced_error(a, vec)
    assert got.scale == wsc and np.array_equal(got.data, want)
