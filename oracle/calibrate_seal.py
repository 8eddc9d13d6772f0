"""Time the oracle port against the real SEAL-4.1-bs on the same core --
MEASUREMENT INFRASTRUCTURE.  The port (nexus_oracle.c through pyoracle) is the
CPU baseline that travels to the GPU machine; this records how its per-operation
cost compares with SEAL's (built from the NEXUS tree by oracle/build_ref.py,
HEXL off) at the bootstrap's N = 2^16 chain, one thread each:

  relinearize at 31 limbs   Evaluator::relinearize_inplace (evaluator.cpp:1345-1400,
                            the key switch of evaluator.cpp:2724-3022)
  rescale at 31 limbs       Evaluator::rescale_to_next_inplace (evaluator.cpp:1682)
  encode at 31 limbs        CKKSEncoder::encode of 32768 complex slots (ckks.h:457-640)

Writes oracle/seal_calibration.json.  Run where the NEXUS sources are
available:  python oracle/calibrate_seal.py
"""
from __future__ import annotations

import json
import platform
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from oracle import nexus_l3 as L  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from oracle import pyref as pr  # noqa: E402

BOOT_BITS = [51] + [46] * 16 + [51] * 14 + [51]
OUT = Path(__file__).resolve().parent / "seal_calibration.json"


def best(f, reps=3):
    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        f()
        t.append(time.perf_counter() - t0)
    return min(t)


def main():
    assert pr.available(), "SEAL reference build unavailable"
    po.set_threads(1)
    log_n, n = 16, 1 << 16
    qs = po.create_coeff_modulus(n, BOOT_BITS)
    ref = pr.SealRef(log_n, qs, seed=np.arange(1, 9, dtype=np.uint64), hamming_weight=192)
    rk = ref.relin_key()
    oc = po.OracleContext(log_n, qs)
    ev = L.Evaluator(oc, rk, {})
    rng = np.random.default_rng(1)
    l = len(qs) - 1
    ct3 = po.random_residues(rng, (3, l, n), qs[:l])
    ct2 = np.ascontiguousarray(ct3[:2])
    vals = rng.uniform(-1, 1, n // 2) + 1j * rng.uniform(-1, 1, n // 2)
    rows = {}
    checks = {}
    s_relin = best(lambda: ref.relinearize(ct3))
    p_relin = best(lambda: oc.relinearize(ct3, rk))
    checks["relinearize"] = bool(np.array_equal(ref.relinearize(ct3), oc.relinearize(ct3, rk)))
    rows["relinearize_l31"] = (s_relin, p_relin)
    s_rs = best(lambda: ref.rescale(ct2, 2.0 ** 46))
    p_rs = best(lambda: oc.rescale(ct2))
    checks["rescale"] = bool(np.array_equal(ref.rescale(ct2, 2.0 ** 46)[0], oc.rescale(ct2)))
    rows["rescale_l31"] = (s_rs, p_rs)
    s_enc = best(lambda: ref.encode(vals, 2.0 ** 46, l))
    p_enc = best(lambda: ev.encode(vals, 2.0 ** 46, l))
    checks["encode"] = bool(np.array_equal(ref.encode(vals, 2.0 ** 46, l), ev.encode(vals, 2.0 ** 46, l).data))
    rows["encode_l31"] = (s_enc, p_enc)
    doc = {
        "what": "one thread each, best of 3, N=2^16, chain 51 + 16x46 + 14x51 + special 51",
        "host": {"machine": platform.machine(), "processor": platform.processor() or platform.machine()},
        "seal": "SEAL-4.1-bs from the NEXUS tree, built by oracle/build_ref.py (HEXL off)",
        "ops": {k: {"seal_s": round(a, 4), "port_s": round(b, 4), "port_over_seal": round(b / a, 3)}
                for k, (a, b) in rows.items()},
        "words_equal": checks,
    }
    OUT.write_text(json.dumps(doc, indent=1) + "\n")
    print(json.dumps(doc, indent=1))


if __name__ == "__main__":
    main()
