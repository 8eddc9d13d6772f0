"""EvalMod's inverse_deg > 1 branch (ModularReducer.cpp:62-73) on the GPU: the
cosine heap unscaled, plain double angles, then the inverse-sine polynomial
-- its direct degree-3 form and, for degree 5, its odd heap.  The engine's
EvalMod words equal the oracle's (oracle/bootstrap.py) for the same input
and table, the lockstep form equals the single form, and the whole bootstrap
decrypts to its input.  N = 2^13, all 2^12 slots, three more 51-bit
bootstrapping primes than the inverse_deg == 1 chain for the polynomial's
levels."""
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
BITS = [51] + [46] * 2 + [51] * 17 + [51]


@pytest.fixture(scope="module", params=[3, 5])
def env(request, cuda):
    import nexus_gb300 as ng
    from nexus_gb300.operators import Bootstrapper, Evaluator
    from nexus_gb300.remez import load_table
    inverse_deg = request.param
    qs = ng.create_coeff_modulus(N, BITS)
    ctx = ng.Context(LOG_N, qs)
    sk = ctx.keygen_secret(seed=51, hamming_weight=192)
    rk = ctx.keygen_relin(sk, seed=52)
    steps = B.rot_key_steps_3(LOG_NH, LOG_NH)
    gks = {ctx.galois_elt(st): ctx.keygen_galois(sk, ctx.galois_elt(st), seed=53 + i) for i, st in enumerate(steps)}
    ev = Evaluator(ctx, SCALE, rk, gks)
    bs = Bootstrapper(ev, loge=10, logn=LOG_NH, logNh=LOG_NH, L=len(BITS) - 2, final_scale=SCALE, boundary_K=25,
                      sin_cos_deg=59, scale_factor=2, inverse_deg=inverse_deg)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    table = load_table(inverse_deg=inverse_deg)
    oev = L.Evaluator(po.OracleContext(LOG_N, qs), to_host(rk), {e: to_host(k) for e, k in gks.items()})
    obs = B.Bootstrapper(oev, 10, LOG_NH, LOG_NH, len(BITS) - 2, SCALE, 25, 59, 2, inverse_deg, table)
    return ctx, sk, bs, obs


def _input(ctx, sk, seed):
    import torch
    from nexus_gb300.operators import Ciphertext
    vals = np.random.default_rng(seed).uniform(-1, 1, N // 2)
    top = len(ctx.moduli) - 1
    pt = torch.empty((top, N), dtype=torch.int64, device="cuda")
    ctx.encode(vals, SCALE, top, pt)
    ct = ctx.encrypt_symmetric(sk, pt, top, seed)
    low = to_host(ct)[:, :1, :].copy()
    return vals, Ciphertext.from_numpy(ctx, low, SCALE)


def test_evalmod_matches_oracle(env):
    from nexus_gb300.operators import (BOOT_COEFFTOSLOT, BOOT_MODRAISE, BOOT_MODULAR_REDUCTION,
                                       BOOT_SET_INITIAL_SCALE, Ciphertext)
    ctx, sk, bs, obs = env
    _, x = _input(ctx, sk, 61)
    bs.stage(BOOT_SET_INITIAL_SCALE, x)
    bs.stage(BOOT_MODRAISE, x)
    x = Ciphertext.from_numpy(ctx, x.to_numpy(), float(ctx.moduli[0]))
    r1, r2 = bs.stage(BOOT_COEFFTOSLOT, x)
    for r in (r1, r2):
        m, _ = bs.stage(BOOT_MODULAR_REDUCTION, r)
        om = obs.modular_reduction(L.Ct(r.to_numpy(), r.scale))
        assert m.scale == om.scale
        assert np.array_equal(m.to_numpy(), om.data)
    # lockstep EvalMod of both halves: the same words
    b1, _ = bs.stage_batch(BOOT_MODULAR_REDUCTION, [r1, r2])
    s1, _ = bs.stage(BOOT_MODULAR_REDUCTION, r1)
    s2, _ = bs.stage(BOOT_MODULAR_REDUCTION, r2)
    assert np.array_equal(b1[0].to_numpy(), s1.to_numpy()) and np.array_equal(b1[1].to_numpy(), s2.to_numpy())


def test_bootstrap_decrypts_to_input(env):
    from nexus_gb300.operators import Ciphertext
    ctx, sk, bs, _ = env
    vals, x = _input(ctx, sk, 62)
    low = x.to_numpy()
    out = bs.bootstrap_3(Ciphertext.from_numpy(ctx, low, SCALE))
    assert out.scale == SCALE
    dec = ctx.decode(ctx.decrypt(sk, out.to_device()), out.scale).real
    assert np.abs(dec - vals).max() < 2.0 ** -10
    batch = bs.bootstrap_batch([Ciphertext.from_numpy(ctx, low, SCALE),
                                Ciphertext.from_numpy(ctx, low[:, :, ::-1].copy(), SCALE)])
    assert np.array_equal(batch[0].to_numpy(), out.to_numpy())
