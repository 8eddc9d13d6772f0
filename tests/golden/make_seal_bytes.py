"""Generate tests/golden/seal_ciphertext_bytes.npz with the real SEAL-4.1-bs
library: Ciphertext::save (compr_mode none) of two ciphertexts -- a fresh one
at the top level (2 polys x 2 limbs) and a size-3 product dropped to one limb
-- with the words, scales and parms_ids they were saved from.

Run where the NEXUS sources are available (the SEAL build in oracle/_ref
needs them):  python tests/golden/make_seal_bytes.py
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
    s = pr.SealRef(log_n, qs, seed=5)
    rng = np.random.default_rng(9)
    a = s.encrypt(rng.uniform(-1, 1, n // 2), 2.0 ** 30)
    b3 = s.multiply(a, a)[:, :1, :].copy()
    out = {}
    for name, ct, scale in (("a", a, 2.0 ** 30), ("b3", b3, 2.0 ** 60)):
        out[f"{name}_words"] = ct
        out[f"{name}_scale"] = np.array(scale)
        out[f"{name}_pid"] = s.parms_id(ct.shape[1])
        out[f"{name}_bytes"] = np.frombuffer(s.save(ct, scale), dtype=np.uint8)
    np.savez_compressed(Path(__file__).parent / "seal_ciphertext_bytes.npz", **out)


if __name__ == "__main__":
    main()
