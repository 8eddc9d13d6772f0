"""Rotations of one ciphertext by several steps sharing one decomposition.

nexus_rotate_vector_many and its lockstep form must give, for every step,
exactly the words of the ordinary Galois key switch (nexus_apply_galois): on
random ciphertexts (the shared-ModUp path), on a ciphertext whose c1 has a
zero coefficient in coefficient form and on a trivial one (both are
recomputed by the device-enabled fallback launch, in a batch only for the
member concerned), below the level where sharing pays, and for step 0.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu

LOG_N = 13
N = 1 << LOG_N
SCALE = 2.0 ** 40
STEPS = [1, 2, 3, -4, 7]


@pytest.fixture(scope="module")
def env(cuda):
    import nexus_gb300 as ng
    from nexus_gb300.operators import Evaluator
    qs = ng.create_coeff_modulus(N, [51] + [46] * 10 + [51])
    ctx = ng.Context(LOG_N, qs)
    sk = ctx.keygen_secret(seed=5)
    rk = ctx.keygen_relin(sk, seed=6)
    keys = {ctx.galois_elt(s): ctx.keygen_galois(sk, ctx.galois_elt(s), seed=10 + i) for i, s in enumerate(STEPS)}
    ev = Evaluator(ctx, SCALE, rk, keys)
    return ctx, ev, keys, qs


def _check(ctx, ev, keys, data, steps):
    import torch
    from nexus_gb300.operators import Ciphertext
    x = Ciphertext.from_numpy(ctx, data, SCALE)
    outs = ev.rotate_vector_many(x, steps)
    assert np.array_equal(x.to_numpy(), data), "the input must be left unchanged"
    for s, o in zip(steps, outs):
        assert o.scale == SCALE
        if s == 0:
            assert np.array_equal(o.to_numpy(), data)
            continue
        elt = ctx.galois_elt(s)
        d = to_dev(data)
        want = torch.empty_like(d)
        ctx.apply_galois(d, elt, keys[elt], want)
        assert np.array_equal(o.to_numpy(), to_host(want)), s


@pytest.mark.parametrize("limbs", [11, 8])
def test_shared_decomposition_matches_apply_galois(env, limbs):
    ctx, ev, keys, qs = env
    rng = np.random.default_rng(limbs)
    data = po.random_residues(rng, (2, limbs, N), qs[:limbs])
    _check(ctx, ev, keys, data, STEPS + [0])


def test_below_the_sharing_level(env):
    ctx, ev, keys, qs = env
    data = po.random_residues(np.random.default_rng(3), (2, 3, N), qs[:3])
    _check(ctx, ev, keys, data, STEPS)


def test_zero_coefficient_falls_back(env):
    """A zero coefficient of INTT(c1) breaks the shared form; the words must not change."""
    ctx, ev, keys, qs = env
    limbs = 10
    rng = np.random.default_rng(4)
    data = po.random_residues(rng, (2, limbs, N), qs[:limbs])
    oc = po.OracleContext(LOG_N, qs)
    coeff = oc.ntt(data[1], 0, limbs, inverse=True)
    coeff[3, 17] = 0
    data[1] = oc.ntt(coeff, 0, limbs)
    _check(ctx, ev, keys, data, STEPS)


def test_trivial_c1_falls_back(env):
    ctx, ev, keys, qs = env
    limbs = 9
    data = po.random_residues(np.random.default_rng(5), (2, limbs, N), qs[:limbs])
    data[1] = 0
    _check(ctx, ev, keys, data, STEPS)


def test_hoisting_off_gives_the_same_words(env):
    ctx, ev, keys, qs = env
    from nexus_gb300.operators import Ciphertext
    data = po.random_residues(np.random.default_rng(6), (2, 11, N), qs[:11])
    x = Ciphertext.from_numpy(ctx, data, SCALE)
    on = [o.to_numpy() for o in ev.rotate_vector_many(x, STEPS)]
    ev.set_hoisting(False)
    try:
        off = [o.to_numpy() for o in ev.rotate_vector_many(x, STEPS)]
    finally:
        ev.set_hoisting(True)
    assert all(np.array_equal(a, b) for a, b in zip(on, off))


def _zero_at(ctx, qs, data, limb, pos):
    """data with coefficient `pos` of INTT(c1)'s limb `limb` set to zero."""
    oc = po.OracleContext(LOG_N, qs)
    limbs = data.shape[1]
    coeff = oc.ntt(data[1], 0, limbs, inverse=True)
    coeff[limb, pos] = 0
    out = data.copy()
    out[1] = oc.ntt(coeff, 0, limbs)
    return out


def test_lockstep_member_with_a_zero_is_recomputed(env):
    """In a lockstep batch only the member with a zero takes the fallback;
    every member's words equal its own apply_galois."""
    import torch
    from nexus_gb300.operators import Ciphertext
    ctx, ev, keys, qs = env
    limbs = 11
    rng = np.random.default_rng(7)
    datas = [po.random_residues(rng, (2, limbs, N), qs[:limbs]) for _ in range(3)]
    datas[1] = _zero_at(ctx, qs, datas[1], 5, 4000)
    datas[2][1] = 0
    xs = [Ciphertext.from_numpy(ctx, d, SCALE) for d in datas]
    res = ev.rotate_vector_many_batch(xs, STEPS)
    for s, row in zip(STEPS, res):
        elt = ctx.galois_elt(s)
        for d, o in zip(datas, row):
            want = torch.empty_like(to_dev(d))
            ctx.apply_galois(to_dev(d), elt, keys[elt], want)
            assert o.scale == SCALE
            assert np.array_equal(o.to_numpy(), to_host(want)), s


def test_lockstep_matches_single_form(env):
    from nexus_gb300.operators import Ciphertext
    ctx, ev, keys, qs = env
    rng = np.random.default_rng(8)
    datas = [po.random_residues(rng, (2, 9, N), qs[:9]) for _ in range(2)]
    xs = [Ciphertext.from_numpy(ctx, d, SCALE) for d in datas]
    res = ev.rotate_vector_many_batch(xs, STEPS + [0])
    for b, x in enumerate(xs):
        single = ev.rotate_vector_many(x, STEPS + [0])
        for row, o in zip(res, single):
            assert np.array_equal(row[b].to_numpy(), o.to_numpy())
