"""The other forms of the forward NTT (nexus_set_ntt_form): 1, the one-pass
form in which thread-block clusters of N/4096 CTAs hold each limb in
distributed shared memory between the columns and the rows pass, and 2, the
two-pass form whose rows pass takes one row of several limbs of one prime
per CTA.  Each must give the oracle's words at every supported ring degree,
for large and small primes (form 2 with polynomial counts that fill and do
not fill its limb groups), and the key switch (whose ModUp and ModDown feed
the transform through its loaders) must give the same words in every form."""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("log_n,bits", [
    (12, [60, 40, 40, 60]),
    (13, [60, 40, 40, 40, 60]),
    (14, [60] + [40] * 7 + [60]),
    (15, [50, 40, 60]),
    (16, [60] * 3),
    (13, [51, 46, 46, 51, 51]),
    (16, [51] + [46] * 3 + [51] * 2),
])
@pytest.mark.parametrize("form,polys", [(1, 3), (2, 3), (2, 70)])
def test_cluster_forward_matches_oracle(cuda, log_n, bits, form, polys):
    from nexus_gb300 import Context
    n = 1 << log_n
    qs = po.create_coeff_modulus(n, bits)
    ctx = Context(log_n, qs)
    ctx.set_ntt_form(form)
    assert ctx.ntt_form() == form
    oc = po.OracleContext(log_n, qs)
    k = len(qs)
    x = po.random_residues(np.random.default_rng(log_n + 100), (polys, k, n), qs)
    t = to_dev(x)
    ctx.ntt_forward(t, 0, k)
    assert np.array_equal(to_host(t), oc.ntt(x, 0, k, threads=8))
    ctx.ntt_inverse(t, 0, k)
    assert np.array_equal(to_host(t), x)


@pytest.mark.parametrize("bits", [[60, 60], [51, 51]])
def test_cluster_forward_edge_values(cuda, bits):
    from nexus_gb300 import Context
    log_n, n = 16, 1 << 16
    qs = po.create_coeff_modulus(n, bits)
    ctx = Context(log_n, qs)
    ctx.set_ntt_form(1)
    oc = po.OracleContext(log_n, qs)
    x = np.zeros((3, 2, n), dtype=np.uint64)
    for j, q in enumerate(qs):
        x[0, j] = q - 1
        x[1, j, ::2] = q - 1
        x[2, j, 0] = 1
    t = to_dev(x)
    ctx.ntt_forward(t, 0, 2)
    assert np.array_equal(to_host(t), oc.ntt(x, 0, 2))


@pytest.mark.parametrize("log_n,bits,limbs,batch", [
    (16, [51] + [46] * 9 + [51], 9, 3),
    (14, [60] + [40] * 7 + [60], 7, 5),
])
def test_key_switch_same_words_in_every_form(cuda, log_n, bits, limbs, batch):
    import torch
    from nexus_gb300 import Context
    n = 1 << log_n
    qs = po.create_coeff_modulus(n, bits)
    ctx = Context(log_n, qs)
    rng = np.random.default_rng(limbs)
    k = len(qs)
    key = po.random_residues(rng, (k - 1, 2, k, n), qs)
    ct = po.random_residues(rng, (batch, 2, limbs, n), qs[:limbs])
    tgt = po.random_residues(rng, (batch, limbs, n), qs[:limbs])
    dkey = to_dev(key)
    outs = []
    for form in (0, 1, 2):
        ctx.set_ntt_form(form)
        d = to_dev(ct)
        ctx.switch_key_batch(d, to_dev(tgt), dkey)
        outs.append(to_host(d))
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    # and the first ciphertext against the oracle
    oc = po.OracleContext(log_n, qs)
    assert np.array_equal(outs[1][0], oc.switch_key(ct[0], tgt[0], key))
