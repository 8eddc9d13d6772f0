"""The identity behind hoisted rotations, on the CPU oracle (N=2^12).

For the Galois element g, the ModUp of the rotated key-switch target
pi_g(c1) equals pi_g applied to the ModUp of c1 plus (q_j mod q_i) times the
NTT of the automorphism's sign mask -- when INTT(c1) has no zero
coefficient.  The key inner product built from the permuted key and the
per-level correction then equals the inner product of the rotated target,
word for word; with zero coefficients it does not, which is why the engine
falls back to one key switch per step there.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

LOG_N = 12
N = 1 << LOG_N


@pytest.fixture(scope="module")
def env():
    qs = po.create_coeff_modulus(N, [50, 40, 45, 55])
    return qs, po.OracleContext(LOG_N, qs)


def _ntt1(oc, x, p):
    return oc.ntt(np.ascontiguousarray(x, dtype=np.uint64).reshape(1, N), p, p + 1)[0].astype(object)


def _modup(oc, qs, t):
    # D[j][i] = NTT_{p(i)}(t_j mod q_{p(i)}), i in 0..l, p(l) = special prime
    K, l = len(qs), len(qs) - 1
    D = np.empty((l, l + 1), dtype=object)
    for j in range(l):
        for i in range(l + 1):
            p = i if i < l else K - 1
            D[j, i] = _ntt1(oc, np.array([int(v) % qs[p] for v in t[j]], dtype=np.uint64), p)
    return D


def _inner(qs, D, key):
    K, l = len(qs), len(qs) - 1
    P = np.empty((2, l + 1), dtype=object)
    for k in range(2):
        for i in range(l + 1):
            p = i if i < l else K - 1
            P[k, i] = sum(D[j, i] * key[j, k, p].astype(object) for j in range(l)) % qs[p]
    return P


def _hoisted(oc, qs, c1, key, elt):
    K, l = len(qs), len(qs) - 1
    table = po.galois_table_ntt(LOG_N, elt).astype(np.int64)
    D = _modup(oc, qs, oc.ntt(c1, 0, l, inverse=True))
    mask = np.zeros(N, dtype=np.uint64)
    raw = (np.arange(N, dtype=np.int64) * elt) % (2 * N)
    mask[raw[raw >= N] - N] = 1
    M = [_ntt1(oc, mask, p) for p in range(K)]
    kperm = np.zeros_like(key)
    kperm[..., table] = key
    Pt = _inner(qs, D, kperm)
    P = np.empty_like(Pt)
    for k in range(2):
        for i in range(l + 1):
            p = i if i < l else K - 1
            acc = sum((qs[j] % qs[p]) * key[j, k, p].astype(object) for j in range(l)) % qs[p]
            P[k, i] = (Pt[k, i][table] + acc * M[p] % qs[p]) % qs[p]
    return P


def _reference(oc, qs, c1, key, elt):
    l = len(qs) - 1
    table = po.galois_table_ntt(LOG_N, elt).astype(np.int64)
    return _inner(qs, _modup(oc, qs, oc.ntt(c1[:, table], 0, l, inverse=True)), key)


def _equal(a, b):
    return all(np.array_equal(a[k, i], b[k, i]) for k in range(a.shape[0]) for i in range(a.shape[1]))


@pytest.mark.parametrize("step", [1, -3])
def test_shared_decomposition_is_exact(env, step):
    qs, oc = env
    l = len(qs) - 1
    rng = np.random.default_rng(step + 10)
    c1 = po.random_residues(rng, (1, l, N), qs[:l])[0]
    key = po.random_residues(rng, (l, 2, len(qs), N), qs)
    elt = po.galois_elt_from_step(LOG_N, step)
    assert _equal(_hoisted(oc, qs, c1, key, elt), _reference(oc, qs, c1, key, elt))


def test_zero_coefficients_break_it(env):
    qs, oc = env
    l = len(qs) - 1
    rng = np.random.default_rng(7)
    t = po.random_residues(rng, (1, l, N), qs[:l])[0]
    t[:, ::5] = 0
    c1 = oc.ntt(t, 0, l)
    key = po.random_residues(rng, (l, 2, len(qs), N), qs)
    elt = po.galois_elt_from_step(LOG_N, 1)
    assert not _equal(_hoisted(oc, qs, c1, key, elt), _reference(oc, qs, c1, key, elt))
