"""Bootstrapping on the GPU engine against the oracle restatement
(oracle/bootstrap.py), word for word, stage by stage and end to end, plus the
decrypted error of the refreshed ciphertext against the input values.

Parameters follow the reference driver (src/bootstrapping.cpp:33-63) at a
smaller ring: N = 2^13 with all 2^12 slots (the full-slot path), q0 51 bits,
two 46-bit primes, fourteen 51-bit bootstrapping primes, a 51-bit special
prime, sparse secret of Hamming weight 192, K = 25, cosine degree 59, two
double-angle steps, loge = 10, scale 2^46."""
import numpy as np
import pytest

from oracle import bootstrap as B
from oracle import nexus_l3 as L
from oracle import pyoracle as po
from tests.util import to_host

pytestmark = pytest.mark.gpu

LOG_N = 13
N = 1 << LOG_N
LOG_NH = LOG_N - 1
SCALE = 2.0 ** 46
BITS = [51] + [46] * 2 + [51] * 14 + [51]
PARAMS = dict(loge=10, logn=LOG_NH, logNh=LOG_NH, L=len(BITS) - 2, final_scale=SCALE, boundary_K=25,
              sin_cos_deg=59, scale_factor=2, inverse_deg=1)


@pytest.fixture(scope="module")
def env(cuda):
    import nexus_gb300 as ng
    from nexus_gb300.operators import Bootstrapper, Evaluator
    from nexus_gb300.remez import load_table
    qs = ng.create_coeff_modulus(N, BITS)
    ctx = ng.Context(LOG_N, qs)
    sk = ctx.keygen_secret(seed=41, hamming_weight=192)
    rk = ctx.keygen_relin(sk, seed=42)
    steps = B.rot_key_steps_3(LOG_NH, LOG_NH)
    gks = {ctx.galois_elt(st): ctx.keygen_galois(sk, ctx.galois_elt(st), seed=43 + i) for i, st in enumerate(steps)}
    ev = Evaluator(ctx, SCALE, rk, gks)
    bs = Bootstrapper(ev, **PARAMS)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    table = load_table()
    oev = L.Evaluator(po.OracleContext(LOG_N, qs), to_host(rk), {e: to_host(k) for e, k in gks.items()})
    obs = B.Bootstrapper(oev, PARAMS["loge"], LOG_NH, LOG_NH, PARAMS["L"], SCALE, 25, 59, 2, 1, table)
    obs.generate_LT_coefficient_3()
    return ctx, sk, bs, obs, steps


def _input(ctx, sk, seed):
    """Encrypt U(-1, 1) slots at the top level and keep the q0 limb only."""
    import torch
    from nexus_gb300.operators import Ciphertext
    vals = np.random.default_rng(seed).uniform(-1, 1, N // 2)
    top = len(ctx.moduli) - 1
    pt = torch.empty((top, N), dtype=torch.int64, device="cuda")
    ctx.encode(vals, SCALE, top, pt)
    ct = ctx.encrypt_symmetric(sk, pt, top, seed)
    low = to_host(ct)[:, :1, :].copy()
    return vals, Ciphertext.from_numpy(ctx, low, SCALE), L.Ct(low, SCALE)


def _same(eng, orc):
    assert eng.scale == orc.scale
    assert np.array_equal(eng.to_numpy(), orc.data)


def _decrypt(ctx, sk, ct):
    return ctx.decode(ctx.decrypt(sk, ct.to_device()), ct.scale).real


def test_rotation_steps_match(env):
    ctx, sk, bs, obs, steps = env
    assert bs.rotation_steps(LOG_NH) == steps


def test_stages_match_oracle(env):
    from nexus_gb300.operators import (BOOT_COEFFTOSLOT, BOOT_MODRAISE, BOOT_MODULAR_REDUCTION,
                                       BOOT_SET_INITIAL_SCALE, BOOT_SLOTTOCOEFF, Ciphertext)
    ctx, sk, bs, obs, _ = env
    _, x, ox = _input(ctx, sk, 5)
    bs.stage(BOOT_SET_INITIAL_SCALE, x)
    obs.initial_scale = ox.scale
    bs.stage(BOOT_MODRAISE, x)
    oraised = obs.modraise_inplace(ox)
    _same(x, oraised)

    q0 = float(ctx.moduli[0])
    x = Ciphertext.from_numpy(ctx, oraised.data, q0)
    oraised.scale = q0
    r1, r2 = bs.stage(BOOT_COEFFTOSLOT, x)
    o1, o2 = obs.coefftoslot_full_3(oraised)
    _same(r1, o1)
    _same(r2, o2)

    m1, _ = bs.stage(BOOT_MODULAR_REDUCTION, r1)
    om1 = obs.modular_reduction(o1)
    _same(m1, om1)
    m2, _ = bs.stage(BOOT_MODULAR_REDUCTION, r2)
    om2 = obs.modular_reduction(o2)
    _same(m2, om2)

    out, _ = bs.stage(BOOT_SLOTTOCOEFF, m1, m2)
    _same(out, obs.slottocoeff_full_3(om1, om2))


def test_lockstep_stages_equal_single_stages(env):
    """nexus_bootstrapper_stage_batch gives each ciphertext the single-stage words."""
    from nexus_gb300.operators import (BOOT_COEFFTOSLOT, BOOT_MODRAISE, BOOT_MODULAR_REDUCTION,
                                       BOOT_SET_INITIAL_SCALE, BOOT_SLOTTOCOEFF, Ciphertext)
    ctx, sk, bs, _, _ = env
    xs = [_input(ctx, sk, 20 + i)[1] for i in range(2)]
    ys = [Ciphertext.from_numpy(ctx, x.to_numpy(), x.scale) for x in xs]
    bs.stage_batch(BOOT_SET_INITIAL_SCALE, xs)
    bs.stage_batch(BOOT_MODRAISE, xs)
    q0 = float(ctx.moduli[0])
    raised = [Ciphertext.from_numpy(ctx, x.to_numpy(), q0) for x in xs]
    c1, c2 = bs.stage_batch(BOOT_COEFFTOSLOT, raised)
    m1, _ = bs.stage_batch(BOOT_MODULAR_REDUCTION, c1)
    m2, _ = bs.stage_batch(BOOT_MODULAR_REDUCTION, c2)
    out, _ = bs.stage_batch(BOOT_SLOTTOCOEFF, m1, m2)
    for k, y in enumerate(ys):
        bs.stage(BOOT_SET_INITIAL_SCALE, y)
        bs.stage(BOOT_MODRAISE, y)
        assert np.array_equal(y.to_numpy(), xs[k].to_numpy())
        y = Ciphertext.from_numpy(ctx, y.to_numpy(), q0)
        s1, s2 = bs.stage(BOOT_COEFFTOSLOT, y)
        assert np.array_equal(s1.to_numpy(), c1[k].to_numpy()) and np.array_equal(s2.to_numpy(), c2[k].to_numpy())
        e1, _ = bs.stage(BOOT_MODULAR_REDUCTION, s1)
        e2, _ = bs.stage(BOOT_MODULAR_REDUCTION, s2)
        assert np.array_equal(e1.to_numpy(), m1[k].to_numpy()) and e1.scale == m1[k].scale
        o, _ = bs.stage(BOOT_SLOTTOCOEFF, e1, e2)
        assert np.array_equal(o.to_numpy(), out[k].to_numpy()) and o.scale == out[k].scale


def test_lockstep_hoisting_falls_back_on_a_trivial_ciphertext(env):
    """A batch in which one ciphertext has c1 = 0 cannot share one exact
    decomposition; the lockstep CoeffToSlot must still give every ciphertext
    the single-form words."""
    from nexus_gb300.operators import BOOT_COEFFTOSLOT, BOOT_MODRAISE, BOOT_SET_INITIAL_SCALE, Ciphertext
    ctx, sk, bs, _, _ = env
    q0 = float(ctx.moduli[0])
    a = _input(ctx, sk, 31)[1]
    trivial = a.to_numpy().copy()
    trivial[1] = 0
    raised = []
    for words in (a.to_numpy(), trivial):
        x = Ciphertext.from_numpy(ctx, words, SCALE)
        bs.stage(BOOT_SET_INITIAL_SCALE, x)
        bs.stage(BOOT_MODRAISE, x)
        raised.append(x.to_numpy())
    xs = [Ciphertext.from_numpy(ctx, w, q0) for w in raised]
    bs.stage_batch(BOOT_SET_INITIAL_SCALE, [a])
    c1, c2 = bs.stage_batch(BOOT_COEFFTOSLOT, xs)
    for k, w in enumerate(raised):
        s1, s2 = bs.stage(BOOT_COEFFTOSLOT, Ciphertext.from_numpy(ctx, w, q0))
        assert np.array_equal(s1.to_numpy(), c1[k].to_numpy()) and np.array_equal(s2.to_numpy(), c2[k].to_numpy())


def test_bootstrap_matches_oracle_and_refreshes(env):
    ctx, sk, bs, obs, _ = env
    vals, x, ox = _input(ctx, sk, 7)
    before = _decrypt(ctx, sk, x)
    out = bs.bootstrap_3(x)
    oout = obs.bootstrap_3(ox)
    _same(out, oout)
    after = _decrypt(ctx, sk, out)
    err = np.abs(after - before)
    assert out.info()[1] >= 2
    assert err.max() < 2.0 ** -12, err.max()


def test_real_pairs_match_oracle_and_refresh(env):
    """nexus_bootstrap_real_batch on three ciphertexts: the first two share
    one bootstrap (c0 + X^(N/2) c1, split by a conjugation) and the third is
    refreshed alone; every word equals the oracle's restatement
    (oracle/bootstrap.py::bootstrap_real_pair) and every output decrypts to
    its own input within a single bootstrap's error."""
    from oracle import bootstrap as OBS
    ctx, sk, bs, obs, _ = env
    ins = [_input(ctx, sk, 40 + i) for i in range(3)]
    before = [_decrypt(ctx, sk, x) for _, x, _ in ins]
    outs = bs.bootstrap_real_batch([x for _, x, _ in ins])
    want = list(OBS.bootstrap_real_pair(obs, ins[0][2].copy(), ins[1][2].copy())) + [obs.bootstrap_3(ins[2][2].copy())]
    for got, o in zip(outs, want):
        _same(got, o)
    for b, out in zip(before, outs):
        err = np.abs(_decrypt(ctx, sk, out) - b)
        assert err.max() < 2.0 ** -12, err.max()


def test_second_bootstrap_reuses_encoded_diagonals(env):
    ctx, sk, bs, obs, _ = env
    _, x1, _ = _input(ctx, sk, 9)
    _, x2, _ = _input(ctx, sk, 9)
    a = bs.bootstrap_3(x1)
    cached = bs.cached_plaintexts()
    assert cached > 0
    b = bs.bootstrap_3(x2)
    assert bs.cached_plaintexts() == cached
    assert np.array_equal(a.to_numpy(), b.to_numpy())


def test_batched_bootstrap_equals_single(env):
    """The lockstep form gives every ciphertext the single form's words."""
    ctx, sk, bs, obs, _ = env
    ins = [_input(ctx, sk, 20 + i) for i in range(3)]
    batch = bs.bootstrap_batch([x for _, x, _ in ins])
    for (_, x, _), got in zip(ins, batch):
        want = bs.bootstrap_3(x)
        assert got.scale == want.scale
        assert np.array_equal(got.to_numpy(), want.to_numpy())
    one = bs.bootstrap_batch([_input(ctx, sk, 20)[1]])[0]
    assert np.array_equal(one.to_numpy(), batch[0].to_numpy())


def test_batched_bootstrap_rejects_mixed_scales(env):
    from nexus_gb300._lib import NexusError
    from nexus_gb300.operators import Ciphertext
    ctx, sk, bs, obs, _ = env
    _, x, ox = _input(ctx, sk, 30)
    y = Ciphertext.from_numpy(ctx, ox.data, SCALE * 2)
    with pytest.raises(NexusError, match="share one scale"):
        bs.bootstrap_batch([x, y])


def test_bootstrap_rejects_higher_level(env):
    from nexus_gb300._lib import NexusError
    from nexus_gb300.operators import Ciphertext
    ctx, sk, bs, obs, _ = env
    data = np.zeros((2, 2, N), dtype=np.uint64)
    with pytest.raises(NexusError, match="lowest level"):
        bs.bootstrap_3(Ciphertext.from_numpy(ctx, data, SCALE))


@pytest.fixture(scope="module")
def sparse_env(cuda):
    """The sparse-slot path (bootstrap_sparse_3): 2^11 distinct slots repeating
    across the 2^12 slots, as the reference driver (src/bootstrapping.cpp) runs it."""
    import nexus_gb300 as ng
    from nexus_gb300.operators import Bootstrapper, Evaluator
    from nexus_gb300.remez import load_table
    logn = LOG_NH - 1
    qs = ng.create_coeff_modulus(N, BITS)
    ctx = ng.Context(LOG_N, qs)
    sk = ctx.keygen_secret(seed=51, hamming_weight=192)
    rk = ctx.keygen_relin(sk, seed=52)
    steps = B.rot_key_steps_3(logn, LOG_NH)
    gks = {ctx.galois_elt(st): ctx.keygen_galois(sk, ctx.galois_elt(st), seed=53 + i) for i, st in enumerate(steps)}
    ev = Evaluator(ctx, SCALE, rk, gks)
    params = dict(PARAMS, logn=logn)
    bs = Bootstrapper(ev, **params)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    oev = L.Evaluator(po.OracleContext(LOG_N, qs), to_host(rk), {e: to_host(k) for e, k in gks.items()})
    obs = B.Bootstrapper(oev, 10, logn, LOG_NH, PARAMS["L"], SCALE, 25, 59, 2, 1, load_table())
    obs.generate_LT_coefficient_3()
    return ctx, sk, bs, obs, steps, logn


def test_sparse_bootstrap_matches_oracle(sparse_env):
    import torch
    from nexus_gb300.operators import Ciphertext
    ctx, sk, bs, obs, steps, logn = sparse_env
    assert bs.rotation_steps(LOG_NH) == steps
    sparse = np.random.default_rng(61).uniform(-1, 1, 1 << logn)
    vals = np.resize(sparse, N // 2)
    top = len(ctx.moduli) - 1
    pt = torch.empty((top, N), dtype=torch.int64, device="cuda")
    ctx.encode(vals, SCALE, top, pt)
    low = to_host(ctx.encrypt_symmetric(sk, pt, top, 62))[:, :1, :].copy()
    x = Ciphertext.from_numpy(ctx, low, SCALE)
    batch = bs.bootstrap_batch([x])[0]
    out = bs.bootstrap_3(x)
    _same(out, obs.bootstrap_3(L.Ct(low, SCALE)))
    assert np.array_equal(batch.to_numpy(), out.to_numpy())
    err = np.abs(_decrypt(ctx, sk, out) - vals)
    assert err.max() < 2.0 ** -12, err.max()


def test_argmax_matches_oracle(cuda):
    """ArgmaxEvaluator (src/argmax.cpp) with a bootstrap per round, on the
    reference's argmax parameters scaled to N=2^12 (sparse slots 2^(logN-2),
    q0 51 bits, 17 x 46-bit, 14 x 51-bit, special 58 bits)."""
    import torch
    import nexus_gb300 as ng
    from nexus_gb300.operators import Bootstrapper, Ciphertext, Evaluator
    from nexus_gb300.remez import load_table
    log_n, length = 12, 4
    n, log_nh = 1 << log_n, log_n - 1
    logn = log_n - 2
    qs = ng.create_coeff_modulus(n, [51] + [46] * 17 + [51] * 14 + [58])
    ctx = ng.Context(log_n, qs)
    sk = ctx.keygen_secret(seed=71, hamming_weight=192)
    rk = ctx.keygen_relin(sk, seed=72)
    steps = B.rot_key_steps_3(logn, log_nh) + [-length]
    gks = {ctx.galois_elt(st): ctx.keygen_galois(sk, ctx.galois_elt(st), seed=73 + i) for i, st in enumerate(steps)}
    ev = Evaluator(ctx, SCALE, rk, gks)
    bs = Bootstrapper(ev, 10, logn, log_nh, len(qs) - 2, SCALE, 25, 59, 2, 1)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    sparse = np.zeros(1 << logn)
    sparse[:length] = [0.1, 0.7, -0.3, 0.2]
    vals = np.resize(sparse, n // 2)
    top = len(qs) - 1
    pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
    ctx.encode(vals, SCALE, top, pt)
    words = to_host(ctx.encrypt_symmetric(sk, pt, top, 74))
    out = bs.argmax(Ciphertext.from_numpy(ctx, words, SCALE), length)
    oev = L.Evaluator(po.OracleContext(log_n, qs), to_host(rk), {e: to_host(k) for e, k in gks.items()})
    obs = B.Bootstrapper(oev, 10, logn, log_nh, len(qs) - 2, SCALE, 25, 59, 2, 1, load_table())
    obs.generate_LT_coefficient_3()
    want = L.argmax(L.CKKSEvaluator(oev, SCALE), obs, L.Ct(words, SCALE), length)
    _same(out, want)
    dec = _decrypt(ctx, sk, out)[:length]
    assert np.argmax(dec) == 1 and dec[1] > 1.5 and np.all(np.abs(np.delete(dec, 1)) < 0.5)
    # the lockstep form over two ciphertexts gives each the single form's words
    other = to_host(ctx.encrypt_symmetric(sk, pt, top, 75))
    xs = [Ciphertext.from_numpy(ctx, words, SCALE), Ciphertext.from_numpy(ctx, other, SCALE)]
    outs = bs.argmax_batch(xs, length)
    _same(outs[0], want)
    single = bs.argmax(Ciphertext.from_numpy(ctx, other, SCALE), length)
    assert np.array_equal(outs[1].to_numpy(), single.to_numpy()) and outs[1].scale == single.scale
