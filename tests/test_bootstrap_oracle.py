"""Bootstrapping on the CPU: the oracle restatement (oracle/bootstrap.py), the
committed EvalMod table (nexus_gb300/remez.py) and the engine's host-side LT
diagonals.

* The engine's diagonals (nexus_lt_coefficients_3, host code) equal the
  oracle's bit for bit.
* The three-level CoeffToSlot / SlotToCoeff diagonals are mutually inverse
  when applied as the BSGS transforms apply them (a plaintext simulation).
* The EvalMod heap reassembles the minimax cosine, the cosine meets its
  levelled error on all 2K-1 intervals, and cosine + double angles give
  x - round(x).
* With SEAL's own keys (where the SEAL reference build exists), the oracle's
  bootstrap decrypts to its input."""
import math

import numpy as np
import pytest

from oracle import bootstrap as B

K = 25


def test_giantstep_and_babycount():
    from nexus_gb300.remez import babycount
    assert [B.giantstep(m) for m in (3, 7, 16, 31, 32, 63)] == [1, 2, 4, 4, 4, 7]
    assert babycount(59) == (8, 3)


def test_rotation_steps():
    s = B.rot_key_steps_3(12, 12)
    assert s[:13] == [0] + [1 << i for i in range(12)]
    assert len(set(s)) == len(s)
    assert all(0 <= x < 4096 for x in s)


@pytest.mark.parametrize("logn,log_nh", [(12, 12), (13, 13), (11, 12), (9, 12)])
def test_engine_diagonals_equal_oracle(logn, log_nh):
    from nexus_gb300.operators import lt_coefficients_3
    orig, inv = B.gen_orig_coeff(logn)
    if logn == log_nh:
        mine = list(B.gen_fft_coeff_3_full(logn, orig)) + list(B.gen_invfft_coeff_3_full(logn, inv, K))
    else:
        mine = list(B.gen_fft_coeff_3_sparse(logn, orig)) + list(B.gen_invfft_coeff_3_sparse(logn, log_nh, inv, K))
    for which, diags in enumerate(mine):
        eng = lt_coefficients_3(logn, log_nh, K, which)
        assert eng.shape[0] == len(diags)
        for i, (re, im) in enumerate(diags):
            assert np.array_equal(eng[i, :len(re), 0].view(np.uint64), re.view(np.uint64)), (which, i)
            assert np.array_equal(eng[i, :len(re), 1].view(np.uint64), im.view(np.uint64)), (which, i)


def _rot(v, s):
    return np.roll(v, -s)


def _bsgs(v, diags, t, step):
    return sum(diags[p + t] * _rot(v, p * step) for p in range(-t, t + 1))


def _rbsgs(v, diags, t, step):
    return sum(diags[p] * _rot(v, p * step) for p in range(t + 1))


def test_lt_levels_are_mutually_inverse():
    logn = 12
    n = 1 << logn
    orig, inv = B.gen_orig_coeff(logn)
    f1, f2, f3 = [[r + 1j * i for r, i in lvl] for lvl in B.gen_fft_coeff_3_full(logn, orig)]
    i1, i2, i3 = [[r + 1j * i for r, i in lvl] for lvl in B.gen_invfft_coeff_3_full(logn, inv, K)]
    d1, d2, d3 = B.split3_inv(logn)
    z = np.random.default_rng(3).standard_normal(n) + 1j * np.random.default_rng(4).standard_normal(n)
    w = _rbsgs(z, i1, (1 << d1) - 1, 1 << (logn - d1))
    w = _bsgs(w, i2, (1 << d2) - 1, 1 << (logn - d1 - d2))
    w = _bsgs(w, i3, (1 << d3) - 1, 1)
    r1 = w + np.conj(w)
    r2 = -1j * w + np.conj(-1j * w)
    assert np.abs(r1.imag).max() < 1e-12 and np.abs(r2.imag).max() < 1e-12
    e1, e2, e3 = B.split3_fwd(logn)
    u = K * (r1 + 1j * r2)
    u = _bsgs(u, f1, (1 << e1) - 1, 1)
    u = _bsgs(u, f2, (1 << e2) - 1, 1 << e1)
    u = _rbsgs(u, f3, (1 << e3) - 1, 1 << (e1 + e2))
    assert np.abs(u - z).max() < 1e-9 * np.abs(z).max()


def _cheb_t(deg, t):
    return np.polynomial.chebyshev.chebval(t, [0] * deg + [1])


def test_evalmod_table():
    from nexus_gb300.remez import load_table
    tb = load_table()
    nodes = tb["nodes"]
    degs = {i: len(c) - 1 for i, c in nodes.items()}
    assert degs == {0: 59, 1: 27, 2: 31, 3: 11, 4: 15, 5: 15, 6: 15, 7: 3, 8: 7, 9: 7, 10: 7, 11: 7, 12: 7, 13: 7,
                    14: 7}
    s = tb["scale_inverse_coeff"]
    assert s == math.sqrt(math.sqrt(float.fromhex(tb["arcsin_c1"])))
    w = 2.0 ** -tb["loge"]
    xs = np.concatenate([np.linspace(i - w, i + w, 41) for i in range(-(K - 1), K)])
    t = xs / K

    def heap_value(i, g):
        if i >= 7:
            return np.polynomial.chebyshev.chebval(t, nodes[i])
        left, right = 2 * i + 1, 2 * i + 2
        return heap_value(left, g + 1) * _cheb_t(8 << (2 - g), t) + heap_value(right, g + 1)

    p = heap_value(0, 0)
    direct = np.polynomial.chebyshev.chebval(t, nodes[0])
    assert np.abs(p - direct).max() < 1e-11
    cos_cheb = [float.fromhex(c) for c in tb["cos_cheb"]]
    target = np.cos(2 * np.pi * (xs - 0.25) / 4)
    approx_err = np.abs(np.polynomial.chebyshev.chebval(t, cos_cheb) - target).max()
    assert approx_err <= tb["cos_levelled_error"] * 1.01 + 1e-15
    assert np.abs(direct - s * target).max() <= s * tb["cos_levelled_error"] * 1.01 + 1e-15
    # two scaled double angles: s^4 cos(2 pi (x - 1/4)) = c1 sin(2 pi x) ~ x - round(x)
    y, cs = direct, s
    for _ in range(tb["double_angle"]):
        cs = cs * cs
        y = 2 * y * y - cs
    assert np.abs(y - (xs - np.round(xs))).max() < 1e-8


@pytest.mark.parametrize("logn", [12, 11])
def test_oracle_bootstrap_decrypts_to_input(logn):
    """Full-slot (logn = logNh) and sparse-slot (logn < logNh, slots repeating
    with period 2^logn as in src/bootstrapping.cpp:139-141) bootstraps."""
    from oracle import nexus_l3 as L
    from oracle import pyoracle as po
    from oracle import pyref as pr
    from nexus_gb300.remez import load_table
    if not pr.available():
        pytest.skip("SEAL reference build unavailable")
    log_n = 13
    n = 1 << log_n
    qs = po.create_coeff_modulus(n, [51] + [46] * 2 + [51] * 14 + [51])
    steps = B.rot_key_steps_3(logn, log_n - 1)
    s = pr.SealRef(log_n, qs, seed=7, hamming_weight=192, steps=steps)
    ev = L.Evaluator(po.OracleContext(log_n, qs), s.relin_key(),
                     {s.galois_elt(st): s.galois_key(s.galois_elt(st)) for st in steps})
    bs = B.Bootstrapper(ev, 10, logn, log_n - 1, len(qs) - 2, 2.0 ** 46, K, 59, 2, 1, load_table())
    bs.generate_LT_coefficient_3()
    sparse = np.random.default_rng(1).uniform(-1, 1, 1 << logn)
    vals = np.resize(sparse, n // 2)
    ct = ev.mod_switch_to(L.Ct(s.encrypt(vals, 2.0 ** 46), 2.0 ** 46), 1)
    out = bs.bootstrap_3(ct)
    assert out.scale == 2.0 ** 46
    err = np.abs(s.decrypt(out.data, out.scale) - vals)
    assert err.max() < 2.0 ** -12


def test_oracle_real_pair_bootstrap_decrypts_to_both_inputs():
    """Two ciphertexts of real values refreshed by one full-slot bootstrap_3
    of c0 + X^(N/2) c1 (scale doubled), split by a conjugation
    (bootstrap_real_pair): with SEAL's keys each output decrypts to its own
    input within a single bootstrap's error."""
    from oracle import nexus_l3 as L
    from oracle import pyoracle as po
    from oracle import pyref as pr
    from nexus_gb300.remez import load_table
    if not pr.available():
        pytest.skip("SEAL reference build unavailable")
    log_n = 13
    n = 1 << log_n
    qs = po.create_coeff_modulus(n, [51] + [46] * 2 + [51] * 14 + [51])
    steps = B.rot_key_steps_3(log_n - 1, log_n - 1)
    s = pr.SealRef(log_n, qs, seed=9, hamming_weight=192, steps=steps)
    ev = L.Evaluator(po.OracleContext(log_n, qs), s.relin_key(),
                     {s.galois_elt(st): s.galois_key(s.galois_elt(st)) for st in steps})
    bs = B.Bootstrapper(ev, 10, log_n - 1, log_n - 1, len(qs) - 2, 2.0 ** 46, K, 59, 2, 1, load_table())
    bs.generate_LT_coefficient_3()
    rng = np.random.default_rng(3)
    vals = [rng.uniform(-1, 1, n // 2) for _ in range(2)]
    cts = [ev.mod_switch_to(L.Ct(s.encrypt(v, 2.0 ** 46), 2.0 ** 46), 1) for v in vals]
    outs = B.bootstrap_real_pair(bs, cts[0], cts[1])
    for v, out in zip(vals, outs):
        assert out.scale == 2.0 ** 46
        err = np.abs(s.decrypt(out.data, out.scale) - v)
        assert err.max() < 2.0 ** -12, err.max()


def test_oddbabycount():
    from nexus_gb300.remez import oddbabycount
    # common/func.cpp:95-118, worked by hand for 5 and 7
    assert oddbabycount(5) == (2, 2) and oddbabycount(7) == (4, 1)
    assert oddbabycount(15) == (4, 2) and oddbabycount(31) == (8, 2)


@pytest.mark.parametrize("inverse_deg", [3, 5])
def test_evalmod_inverse_sine_tables(inverse_deg):
    """inverse_deg > 1: the cosine stays unscaled, the inverse-sine polynomial
    (power basis, and its odd heap above degree 3) follows the plain double
    angles, and the composition is x - round(x)."""
    from nexus_gb300.remez import load_table
    tb = load_table(inverse_deg=inverse_deg)
    inv = tb["inverse"]
    assert inv["deg"] == inverse_deg and len(inv["power"]) == inverse_deg + 1
    assert tb["scale_inverse_coeff"] == 1.0
    base = load_table()
    assert tb["cos_cheb"] == base["cos_cheb"]
    w = 2.0 ** -tb["loge"]
    xs = np.concatenate([np.linspace(i - w, i + w, 41) for i in range(-(K - 1), K)])
    y = np.polynomial.chebyshev.chebval(xs / K, tb["nodes"][0])
    assert np.abs(y - np.cos(2 * np.pi * (xs - 0.25) / 4)).max() <= tb["cos_levelled_error"] * 1.01 + 1e-15
    for _ in range(tb["double_angle"]):
        y = 2 * y * y - 1.0
    p = np.polynomial.polynomial.polyval(y, inv["power"])
    assert np.abs(p - (xs - np.round(xs))).max() < 1e-8
    # odd polynomial: the even coefficients vanish below any ciphertext scale
    assert all(abs(c) < 1e-60 for c in inv["power"][0::2])
    if inverse_deg > 3:
        k, m = inv["heap_k"], inv["heap_m"]
        nodes = inv["nodes"]
        first = (1 << m) - 1

        def heap_value(i, g, t):
            if i >= first:
                return np.polynomial.chebyshev.chebval(t, nodes[i]) if i in nodes else 0.0
            left, right = 2 * i + 1, 2 * i + 2
            if left not in nodes:
                return heap_value(right, g + 1, t)
            return heap_value(left, g + 1, t) * _cheb_t((k << m) >> (g + 1), t) + heap_value(right, g + 1, t)

        t = np.linspace(-0.01, 0.01, 101)
        assert np.abs(heap_value(0, 0, t) - np.polynomial.polynomial.polyval(t, inv["power"])).max() < 1e-15


@pytest.mark.parametrize("inverse_deg", [3, 5])
def test_oracle_bootstrap_with_inverse_sine(inverse_deg):
    """ModularReducer's inverse_deg > 1 branch (ModularReducer.cpp:62-73) in a
    full-slot bootstrap with SEAL's keys: the refreshed ciphertext decrypts
    to the input (the chain has three more bootstrapping primes for the
    polynomial's levels)."""
    from oracle import nexus_l3 as L
    from oracle import pyoracle as po
    from oracle import pyref as pr
    from nexus_gb300.remez import load_table
    if not pr.available():
        pytest.skip("SEAL reference build unavailable")
    log_n, logn = 13, 12
    n = 1 << log_n
    qs = po.create_coeff_modulus(n, [51] + [46] * 2 + [51] * 17 + [51])
    steps = B.rot_key_steps_3(logn, log_n - 1)
    s = pr.SealRef(log_n, qs, seed=9, hamming_weight=192, steps=steps)
    ev = L.Evaluator(po.OracleContext(log_n, qs), s.relin_key(),
                     {s.galois_elt(st): s.galois_key(s.galois_elt(st)) for st in steps})
    bs = B.Bootstrapper(ev, 10, logn, log_n - 1, len(qs) - 2, 2.0 ** 46, K, 59, 2, inverse_deg,
                        load_table(inverse_deg=inverse_deg))
    bs.generate_LT_coefficient_3()
    vals = np.random.default_rng(2).uniform(-1, 1, n // 2)
    ct = ev.mod_switch_to(L.Ct(s.encrypt(vals, 2.0 ** 46), 2.0 ** 46), 1)
    out = bs.bootstrap_3(ct)
    assert out.scale == 2.0 ** 46
    assert np.abs(s.decrypt(out.data, out.scale) - vals).max() < 2.0 ** -12
