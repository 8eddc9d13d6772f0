"""Generate tests/golden/bert_digests.json: SHA-256 digests of the oracle's
words at every stage of the encrypted BERT encoder layer (oracle/bert.py) at
a reduced size: N = 2^13, 128 token slots per feature block (32 blocks per
ciphertext: 2 hidden, 2 head-layout and 5 FFN ciphertexts), hidden 64 =
2 heads x 32, FFN 160, two lanes with requests of 40 | 8 + 32 tokens (the
second copies of the 40- and 32-token requests reach the upper half of the
block), on the chain 51 + 19x46 + 14x51 + special 51 with the sparse secret
(h = 192), two ciphertexts per bootstrap (boot_pack) and the token fold
(Q, K and the post-attention activations two per ciphertext).  Keys and encryptions come from the real SEAL-4.1-bs with one
seeded Blake2xbPRNG factory, so the engine can make them again on the GPU
from the seed (tests/test_bert_gpu.py).

Run where the NEXUS sources are available (oracle/_ref needs them):
    python tests/golden/make_bert_digests.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))

from make_bench_digests import SealKeys, seed8  # noqa: E402
from nexus_gb300 import bert as NB  # noqa: E402  (input packing, weights, FP64 reference: numpy only)
from oracle import bert as OB  # noqa: E402
from oracle import bootstrap as B  # noqa: E402
from oracle import nexus_l3 as L  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from oracle import pyref as pr  # noqa: E402

OUT = Path(__file__).parent / "bert_digests.json"

CASE = dict(log_n=13, bits=[51] + [46] * 19 + [51] * 14 + [51], seed=seed8(500), hamming_weight=192,
            scale_log2=46, loge=10, boundary_K=25, sin_cos_deg=59, scale_factor=2, inverse_deg=1,
            hidden=64, heads=2, head_dim=32, ffn=160, T=128, lanes=[[[0, 40]], [[0, 8], [16, 32]]],
            boot_shrink=1.0, boot_pack=True, token_fold=True, weight_seed=7, token_seed=8)


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def shape_of(c):
    return NB.BertShape(hidden=c["hidden"], heads=c["heads"], head_dim=c["head_dim"], ffn=c["ffn"], T=c["T"],
                        lanes=[[tuple(r) for r in lane] for lane in c["lanes"]], boot_shrink=c["boot_shrink"],
                        boot_pack=c["boot_pack"], token_fold=c["token_fold"])


def inputs(c):
    """Weights and each lane's per-request tokens, seeded."""
    sh = shape_of(c)
    w = NB.random_weights(sh, np.random.default_rng(c["weight_seed"]))
    rng = np.random.default_rng(c["token_seed"])
    tokens = [[rng.normal(0, 1, (Lr, sh.hidden)) for (_, Lr) in lane] for lane in sh.lanes]
    return sh, w, tokens


def main():
    assert pr.available(), "SEAL reference build unavailable"
    po.set_threads(os.cpu_count() or 1)
    c = CASE
    t0 = time.time()
    n = 1 << c["log_n"]
    qs = po.create_coeff_modulus(n, c["bits"])
    log_nh = c["log_n"] - 1
    sh, w, tokens = inputs(c)
    osh = OB.Shape(n // 2, sh.hidden, sh.heads, sh.head_dim, sh.ffn, sh.T, sh.lanes, sh.boot_shrink, sh.boot_pack,
                   token_fold=sh.token_fold)
    assert osh.folding and (osh.n_hid, osh.n_head, osh.n_ffn) == (2, 2, 5) and osh.copy_shifts == [32, 40]
    keys = SealKeys(c["log_n"], qs, c["seed"], c["hamming_weight"], keep=1000)
    steps = B.rot_key_steps_3(log_nh, log_nh)
    for s in osh.rotation_steps():
        if s not in steps:
            steps.append(s)
    keys.allow(keys.ref.galois_elt(s) for s in steps)
    scale = 2.0 ** c["scale_log2"]
    from nexus_gb300.remez import load_table
    oev = L.Evaluator(po.OracleContext(c["log_n"], qs), keys.ref.relin_key(), keys)
    obs = B.Bootstrapper(oev, c["loge"], log_nh, log_nh, len(qs) - 2, scale, c["boundary_K"], c["sin_cos_deg"],
                         c["scale_factor"], c["inverse_deg"], load_table())
    obs.generate_LT_coefficient_3()
    top = len(qs) - 1
    rec = dict(c, moduli=[str(q) for q in qs], rotation_steps=osh.rotation_steps(), lanes_out=[])
    for lane in range(len(sh.lanes)):
        vecs = NB.pack_lane(sh, n // 2, lane, tokens[lane])
        cts, dig = [], []
        for v in vecs:
            ct = keys.ref.encrypt_ntt(oev.encode(v, scale, top).data, scale, symmetric=True)
            cts.append(L.Ct(ct, scale))
            dig.append(digest(ct))
        trace = {}
        layer = OB.BertLayer(oev, obs, osh, w, lane)
        out = layer.forward(cts, trace)
        lrec = {"input": dig, "stages": {k: [digest(x.data) for x in v] for k, v in trace.items()},
                "output_scale": out[0].scale, "output_limbs": out[0].limbs}
        dec = np.stack([keys.ref.decrypt(x.data, x.scale) for x in out])
        got = NB.unpack_lane(sh, n // 2, lane, dec)
        ref = NB.layer_reference(sh, w, tokens[lane])
        lrec["max_abs_err_vs_fp64_same_approx"] = float(max(np.max(np.abs(g - r)) for g, r in zip(got, ref)))
        rec["lanes_out"].append(lrec)
        print(f"lane {lane}: {time.time() - t0:.0f} s, error {lrec['max_abs_err_vs_fp64_same_approx']:.3g}",
              flush=True)
    rec["seconds"] = round(time.time() - t0, 1)
    OUT.write_text(json.dumps(rec, indent=1) + "\n")


if __name__ == "__main__":
    main()
