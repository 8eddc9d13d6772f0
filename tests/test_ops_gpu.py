"""GPU parity of the CKKS ciphertext operations.

(1) against SEAL's own outputs (tests/golden/ckks_n4096.npz), word for word;
(2) against the CPU oracle on seeded random ciphertexts and keys at N=2^16,
    at every level of an 8-prime chain, plus edge values.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.golden_data import load
from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return load()


@pytest.fixture(scope="module")
def gctx(golden, cuda):
    from nexus_gb300 import Context
    return Context(int(golden["log_n"]), [int(q) for q in golden["moduli"]])


def test_golden_ntt(golden, gctx):
    t = to_dev(golden["ntt_in"])
    gctx.ntt_forward(t, 0, 3)
    assert np.array_equal(to_host(t), golden["ntt_out"])


def test_golden_multiply_relin_rescale(golden, gctx):
    import torch
    a, b = to_dev(golden["ct_a"]), to_dev(golden["ct_b"])
    m = torch.empty((3,) + tuple(a.shape[1:]), dtype=torch.int64, device="cuda")
    gctx.multiply(a, b, m)
    assert np.array_equal(to_host(m), golden["mul3"])
    r = torch.empty_like(a)
    gctx.relinearize(m, to_dev(golden["relin_key"]), r)
    assert np.array_equal(to_host(r), golden["relin"])
    out = torch.empty((2, 1, a.shape[2]), dtype=torch.int64, device="cuda")
    gctx.rescale(r, out)
    assert np.array_equal(to_host(out), golden["rescaled"])


def test_golden_galois(golden, gctx):
    import torch
    a = to_dev(golden["ct_a"])
    e1, em3, e0 = [int(e) for e in golden["galois_elts"]]
    assert gctx.galois_elt(1) == e1 and gctx.galois_elt(-3) == em3 and gctx.galois_elt(0) == e0
    for elt, key, want in ((e1, "galois_key_1", "rot1"), (em3, "galois_key_m3", "rotm3"),
                           (e0, "galois_key_conj", "conj")):
        out = torch.empty_like(a)
        gctx.apply_galois(a, elt, to_dev(golden[key]), out)
        assert np.array_equal(to_host(out), golden[want]), want
    low = to_dev(np.ascontiguousarray(golden["ct_a"][:, :1]))
    out = torch.empty_like(low)
    gctx.apply_galois(low, e1, to_dev(golden["galois_key_1"]), out)
    assert np.array_equal(to_host(out), golden["rot1_low"])


def test_golden_multiply_plain(golden, gctx):
    import torch
    a = to_dev(golden["ct_a"])
    out = torch.empty_like(a)
    gctx.plain_op(a, to_dev(golden["pt"]), 0, out)
    assert np.array_equal(to_host(out), golden["mulplain"])


# ---------------------------------------------------------------- N = 2^16

LOG_N = 16
N = 1 << LOG_N


@pytest.fixture(scope="module")
def big(cuda):
    from nexus_gb300 import Context
    qs = po.create_coeff_modulus(N, [60, 40, 40, 50, 40, 40, 60, 60])
    return Context(LOG_N, qs), po.OracleContext(LOG_N, qs), qs


def _rand_ct(rng, size, limbs, qs):
    return po.random_residues(rng, (size, limbs, N), qs[:limbs])


def _rand_key(rng, qs):
    k = len(qs)
    return po.random_residues(rng, (k - 1, 2, k, N), qs)


@pytest.mark.parametrize("limbs", [7, 4, 1])
def test_switch_key_random(big, limbs):
    ctx, oc, qs = big
    rng = np.random.default_rng(limbs)
    ct = _rand_ct(rng, 2, limbs, qs)
    tgt = _rand_ct(rng, 1, limbs, qs)[0]
    key = _rand_key(rng, qs)
    want = oc.switch_key(ct, tgt, key)
    d = to_dev(ct)
    ctx.switch_key(d, to_dev(tgt), to_dev(key))
    assert np.array_equal(to_host(d), want)


@pytest.fixture(scope="module")
def small(cuda):
    """Every prime below 2^52: the reduction-free NTT and split inner product."""
    from nexus_gb300 import Context
    qs = po.create_coeff_modulus(N, [51, 46, 46, 46, 51, 51, 51, 51])
    return Context(LOG_N, qs), po.OracleContext(LOG_N, qs), qs


@pytest.mark.parametrize("chain", ["big", "small"])
@pytest.mark.parametrize("limbs", [7, 2])
def test_switch_key_batch(request, chain, limbs):
    """nexus_switch_key_batch gives every ciphertext the single-call words."""
    import torch
    ctx, oc, qs = request.getfixturevalue(chain)
    rng = np.random.default_rng(100 + limbs)
    cts = [_rand_ct(rng, 2, limbs, qs) for _ in range(3)]
    tgts = [_rand_ct(rng, 1, limbs, qs)[0] for _ in range(3)]
    key = _rand_key(rng, qs)
    d = to_dev(np.stack(cts))
    t = to_dev(np.stack(tgts))
    ctx.switch_key_batch(d, t, to_dev(key))
    got = to_host(d)
    for b in range(3):
        assert np.array_equal(got[b], oc.switch_key(cts[b], tgts[b], key)), b
    assert np.array_equal(to_host(t), np.stack(tgts)), "targets must be left unchanged"
    with pytest.raises(RuntimeError):
        ctx.switch_key_batch(d, d[:, 0], to_dev(key))
    empty = torch.empty((0, 2, limbs, N), dtype=torch.int64, device="cuda")
    ctx.switch_key_batch(empty, torch.empty((0, limbs, N), dtype=torch.int64, device="cuda"), to_dev(key))


@pytest.mark.parametrize("limbs", [7, 3, 2])
def test_rescale_random(big, limbs):
    import torch
    ctx, oc, qs = big
    rng = np.random.default_rng(100 + limbs)
    ct = _rand_ct(rng, 3, limbs, qs)
    out = torch.empty((3, limbs - 1, N), dtype=torch.int64, device="cuda")
    ctx.rescale(to_dev(ct), out)
    assert np.array_equal(to_host(out), oc.rescale(ct))


def test_multiply_relin_rotate_random(big):
    import torch
    ctx, oc, qs = big
    rng = np.random.default_rng(9)
    limbs = 5
    a, b = _rand_ct(rng, 2, limbs, qs), _rand_ct(rng, 2, limbs, qs)
    key = _rand_key(rng, qs)
    da, db = to_dev(a), to_dev(b)
    m = torch.empty((3, limbs, N), dtype=torch.int64, device="cuda")
    ctx.multiply(da, db, m)
    want3 = oc.multiply(a, b)
    assert np.array_equal(to_host(m), want3)
    r = torch.empty_like(da)
    ctx.relinearize(m, to_dev(key), r)
    assert np.array_equal(to_host(r), oc.relinearize(want3, key))
    for step in (1, -7, 256, 0):
        elt = ctx.galois_elt(step)
        assert elt == po.galois_elt_from_step(LOG_N, step)
        out = torch.empty_like(da)
        ctx.apply_galois(da, elt, to_dev(key), out)
        assert np.array_equal(to_host(out), oc.apply_galois(a, elt, key)), step


def test_elementwise_random(big):
    import torch
    ctx, oc, qs = big
    rng = np.random.default_rng(3)
    limbs = 6
    a, b = _rand_ct(rng, 2, limbs, qs), _rand_ct(rng, 2, limbs, qs)
    pt = _rand_ct(rng, 1, limbs, qs)[0]
    da, db = to_dev(a), to_dev(b)
    out = torch.empty_like(da)
    ctx.add(da, db, out)
    assert np.array_equal(to_host(out), oc.add(a, b))
    ctx.sub(da, db, out)
    assert np.array_equal(to_host(out), oc.sub(a, b))
    ctx.negate(da, out)
    q = np.array(qs[:limbs], dtype=np.uint64).reshape(1, limbs, 1)
    assert np.array_equal(to_host(out), np.where(a == 0, 0, q - a))
    ctx.plain_op(da, to_dev(pt), 0, out)
    assert np.array_equal(to_host(out), oc.multiply_plain(a, pt))


def test_edge_values(big):
    """all-zero and all-(q-1) ciphertexts through key switching and rescale"""
    import torch
    ctx, oc, qs = big
    limbs = 4
    q = np.array(qs[:limbs], dtype=np.uint64).reshape(1, limbs, 1)
    rng = np.random.default_rng(1)
    key = _rand_key(rng, qs)
    for ct in (np.zeros((2, limbs, N), np.uint64), np.broadcast_to(q - np.uint64(1), (2, limbs, N)).copy()):
        d = to_dev(ct)
        ctx.switch_key(d, to_dev(ct[1]), to_dev(key))
        assert np.array_equal(to_host(d), oc.switch_key(ct, ct[1], key))
        out = torch.empty((2, limbs - 1, N), dtype=torch.int64, device="cuda")
        ctx.rescale(to_dev(ct), out)
        assert np.array_equal(to_host(out), oc.rescale(ct))
