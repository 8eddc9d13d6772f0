"""Generate tests/golden/ckks_n4096.npz with the real SEAL-4.1-bs library.

Run where the NEXUS sources are available (the SEAL build in oracle/_ref needs
them):  python tests/golden/make_golden.py

Parameters: N = 4096, CoeffModulus::Create(4096, {50, 40, 50}) -> two data
primes + the special prime, keys from SEAL's KeyGenerator under a seeded
Blake2xb PRNG, values uniform in [-1, 1] from numpy seed 2024, scale 2^30.
Every array is SEAL's own output; the tests compare the oracle and the CUDA
engine against them word for word.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pyoracle as po  # noqa: E402
from oracle import pyref as pr  # noqa: E402


def main():
    assert pr.available(), "SEAL reference build unavailable"
    log_n, n = 12, 1 << 12
    qs = po.create_coeff_modulus(n, [50, 40, 50])
    scale = 2.0 ** 30
    s = pr.SealRef(log_n, qs, seed=77, steps=[0, 1, -3])
    rng = np.random.default_rng(2024)
    va = rng.uniform(-1, 1, n // 2)
    vb = rng.uniform(-1, 1, n // 2)
    vp = rng.uniform(-1, 1, n // 2)
    ct_a = s.encrypt(va, scale)
    ct_b = s.encrypt(vb, scale)
    mul3 = s.multiply(ct_a, ct_b)
    relin = s.relinearize(mul3)
    rescaled, new_scale = s.rescale(relin, scale * scale)
    e1, e3, e0 = s.galois_elt(1), s.galois_elt(-3), s.galois_elt(0)
    rot1 = s.rotate(ct_a, 1)
    rotm3 = s.rotate(ct_a, -3)
    conj = s.conjugate(ct_a)
    rot1_low = s.rotate(np.ascontiguousarray(ct_a[:, :1]), 1)
    pt = s.encode(vp, scale, 2)
    mulplain = s.multiply_plain(ct_a, pt)
    vc = rng.uniform(-1, 1, n // 2) + 1j * rng.uniform(-1, 1, n // 2)
    pt_complex = s.encode(vc, 2.0 ** 35, 2)
    pt_short = s.encode(vp[:100], 2.0 ** 20, 1)
    scalar_vals = np.array([0.0, 1.0, -1.0, 0.5, -3.75, 1e-3, 123.456, -0.011])
    scalar_scales = np.array([2.0 ** 30, 2.0 ** 40, 2.0 ** 45.5, 2.0 ** 20, 2.0 ** 30, 2.0 ** 50, 2.0 ** 30,
                              2.0 ** 60])
    scalar_pts = np.stack([s.encode_scalar(v, sc, 2)[:, 0] for v, sc in zip(scalar_vals, scalar_scales)])
    decoded = s.decode(pt, scale)
    x = po.random_residues(rng, (2, 3, n), qs)
    ntt = np.stack([np.stack([pr.ntt(log_n, qs[j], x[p, j]) for j in range(3)]) for p in range(2)])
    out = Path(__file__).parent / "ckks_n4096.npz"
    np.savez(out, log_n=log_n, moduli=np.array(qs, dtype=np.uint64), scale=scale, new_scale=new_scale,
             values_a=va, values_b=vb, values_p=vp,
             relin_key=s.relin_key(), galois_key_1=s.galois_key(e1), galois_key_m3=s.galois_key(e3),
             galois_key_conj=s.galois_key(e0), galois_elts=np.array([e1, e3, e0], dtype=np.uint32),
             ct_a=ct_a, ct_b=ct_b, mul3=mul3, relin=relin, rescaled=rescaled, rot1=rot1, rotm3=rotm3,
             conj=conj, rot1_low=rot1_low, pt=pt, mulplain=mulplain, ntt_in=x, ntt_out=ntt,
             secret_key=s.secret_key(), values_c=vc, pt_complex=pt_complex, pt_short=pt_short,
             scalar_vals=scalar_vals, scalar_scales=scalar_scales, scalar_pts=scalar_pts, decoded=decoded)
    # one large-ring encode pins the N = 2^16 root table (2^17-th roots of unity)
    log_n2, n2 = 16, 1 << 16
    qs2 = po.create_coeff_modulus(n2, [60, 50, 60])
    s2 = pr.SealRef(log_n2, qs2, seed=1)
    v2 = np.random.default_rng(7).uniform(-1, 1, n2 // 2)
    out2 = Path(__file__).parent / "ckks_encode_n65536.npz"
    np.savez(out2, log_n=log_n2, moduli=np.array(qs2, dtype=np.uint64), values=v2,
             pt=s2.encode(v2, 2.0 ** 40, 2), decoded=s2.decode(s2.encode(v2, 2.0 ** 40, 2), 2.0 ** 40))
    print(out2, out2.stat().st_size)
    print(out, out.stat().st_size)


if __name__ == "__main__":
    main()
