"""GPU parity of the batched NTT against the CPU oracle (bit-exact)."""
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
    # every prime below 2^52: the forward NTT's reduction-free small-prime path
    (13, [51, 46, 46, 51, 51]),
    (16, [51] + [46] * 3 + [51] * 2),
    (14, [52, 52, 30]),
])
def test_ntt_forward_inverse_matches_oracle(cuda, log_n, bits):
    from nexus_gb300 import Context
    n = 1 << log_n
    qs = po.create_coeff_modulus(n, bits)
    ctx = Context(log_n, qs)
    oc = po.OracleContext(log_n, qs)
    assert [int(x) for x in ctx.psi()] == [oc.root(j) for j in range(len(qs))]
    rng = np.random.default_rng(log_n)
    k = len(qs)
    x = po.random_residues(rng, (3, k, n), qs)
    want = oc.ntt(x, 0, k, threads=4)
    t = to_dev(x)
    ctx.ntt_forward(t, 0, k)
    got = to_host(t)
    assert np.array_equal(got, want)
    ctx.ntt_inverse(t, 0, k)
    assert np.array_equal(to_host(t), x)
    # inverse of arbitrary NTT-domain data also matches SEAL's inverse
    y = po.random_residues(rng, (2, k, n), qs)
    t = to_dev(y)
    ctx.ntt_inverse(t, 0, k)
    assert np.array_equal(to_host(t), oc.ntt(y, 0, k, inverse=True, threads=4))


def test_ntt_limb_subrange(cuda):
    from nexus_gb300 import Context
    log_n, n = 14, 1 << 14
    qs = po.create_coeff_modulus(n, [60, 50, 40, 30, 60])
    ctx = Context(log_n, qs)
    oc = po.OracleContext(log_n, qs)
    rng = np.random.default_rng(3)
    x = po.random_residues(rng, (4, 2, n), qs[1:3])
    t = to_dev(x)
    ctx.ntt_forward(t, 1, 3)
    assert np.array_equal(to_host(t), oc.ntt(x, 1, 3))


@pytest.mark.parametrize("bits", [[60, 60], [51, 51]])
def test_ntt_edge_values(cuda, bits):
    """All-zero, all q-1 and single-spike inputs (all q-1 is the largest
    input of the small-prime path too)."""
    from nexus_gb300 import Context
    log_n, n = 16, 1 << 16
    qs = po.create_coeff_modulus(n, bits)
    ctx = Context(log_n, qs)
    oc = po.OracleContext(log_n, qs)
    q = np.array(qs, dtype=np.uint64).reshape(2, 1)
    cases = [np.zeros((2, n), np.uint64), np.broadcast_to(q - np.uint64(1), (2, n)).copy()]
    spike = np.zeros((2, n), np.uint64)
    spike[:, 12345] = 1
    cases.append(spike)
    for x in cases:
        t = to_dev(x)
        ctx.ntt_forward(t, 0, 2)
        assert np.array_equal(to_host(t), oc.ntt(x, 0, 2))


def test_ntt_full_size_round_trip(cuda):
    """The benchmarked NTT shape (N=2^16, 24 x 60-bit primes), 64 ciphertexts x 2 polys:
    INTT(NTT(x)) == x everywhere plus oracle agreement on sampled limbs."""
    import torch
    from nexus_gb300 import Context
    log_n, n = 16, 1 << 16
    qs = po.create_coeff_modulus(n, [60] * 24)
    ctx = Context(log_n, qs)
    g = torch.Generator(device="cuda").manual_seed(5)
    qd = torch.tensor([int(q) for q in qs], dtype=torch.int64, device="cuda").view(1, 24, 1)
    x = torch.randint(0, 2**62, (128, 24, n), generator=g, device="cuda", dtype=torch.int64) % qd
    ref = x.clone()
    ctx.ntt_forward(x, 0, 24)
    sample = to_host(x[17:18])  # one polynomial, all limbs
    ctx.ntt_inverse(x, 0, 24)
    assert torch.equal(x, ref)
    oc = po.OracleContext(log_n, qs)
    assert np.array_equal(sample, oc.ntt(to_host(ref[17:18]), 0, 24, threads=8))
