"""Generate tests/golden/bench_digests.json: SHA-256 digests of the oracle's
output words at the configurations that bench.py measures, with keys and
encryptions made by the real SEAL-4.1-bs from seeded Blake2xbPRNG factories
(every create() call of a factory gets the same 8-word seed), so that the
GPU engine can regenerate every key and input on the device from the seeds
(nexus_seal_*) and compare its own outputs' digests.

Cases:
  keyswitch_n65536_l31  switch_key_inplace (evaluator.cpp:2724-3022) with a
                        SEAL relinearization key on the 32-prime bootstrap
                        chain at 31 limbs, and a rotation by one slot with a
                        SEAL Galois key (apply_galois_inplace, :2563-2665);
  gelu_n16384           GeLUEvaluator::gelu (src/gelu.cpp:5-111) at N=2^14 on
                        the reference chain 58 + 18x40 + 58, one ciphertext of
                        U(-5,5) and one of U(-8,8) slots;
  matmul_n65536         MMEvaluator::matrix_mul (src/matrix_mul.cpp:174-246) at
                        the BERT shape 128x768 . 768x768 + b on 60+40+60; the
                        compressed operand comes from NEXUS's own
                        enc_compress_ciphertext; rows 0, 85 (split across the
                        two compressed ciphertexts) and 127, whose expansion
                        subtrees alone are computed;
  bootstrap_n65536      Bootstrapper::bootstrap_3 (Bootstrapper.cpp:3489-3495)
                        full-slot at N=2^16 on 51 + 16x46 + 14x51 + 51 with
                        the sparse secret (h = 192), K = 25, degree 59, two
                        double angles: every stage's output;
  bert_n65536_qkv       the encrypted BERT-base layer's Q, K and V projections
                        for the 128-token lane at N=2^16 on the layer chain
                        51 + 19x46 + 14x51 + 51, from the inputs bench.py's
                        layer receives (weights and tokens from its seeds).

Digests are over the little-endian bytes of the uint64 arrays in SEAL's
layout.  The oracle's key switch and rescale run on all host cores.

Run where the NEXUS sources are available (the SEAL build in oracle/_ref
needs them):  python tests/golden/make_bench_digests.py [case ...]
"""
from __future__ import annotations

import hashlib
import json
import math
import os
import sys
import time
from collections import OrderedDict
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import bootstrap as B  # noqa: E402
from oracle import nexus_l3 as L  # noqa: E402
from oracle import pyoracle as po  # noqa: E402
from oracle import pyref as pr  # noqa: E402

OUT = Path(__file__).parent / "bench_digests.json"

BOOT_BITS = [51] + [46] * 16 + [51] * 14 + [51]
GELU_BITS = [58] + [40] * 18 + [58]
MM_BITS = [60, 40, 60]
BERT_BITS = [51] + [46] * 19 + [51] * 14 + [51]


def seed8(tag: int) -> list[int]:
    return [int((0x9E3779B97F4A7C15 * (tag + i + 1)) % 2 ** 64) for i in range(8)]


CASES = {
    "keyswitch_n65536_l31": dict(log_n=16, bits=BOOT_BITS, seed=seed8(100), hamming_weight=192, limbs=31,
                                 data_seed=31, rotate_step=1),
    "gelu_n16384": dict(log_n=14, bits=GELU_BITS, seed=seed8(200), hamming_weight=0, scale_log2=40,
                        inputs=[dict(lo=-5.0, hi=5.0, data_seed=777), dict(lo=-8.0, hi=8.0, data_seed=778)]),
    "matmul_n65536": dict(log_n=16, bits=MM_BITS, seed=seed8(300), hamming_weight=0, rows=128, cols=768, out=768,
                          data_seed=2024, pt_scale_log2=40, pack_scale=1e10, check_rows=[0, 85, 127]),
    "bootstrap_n65536": dict(log_n=16, bits=BOOT_BITS, seed=seed8(400), hamming_weight=192, scale_log2=46,
                             data_seed=4096, loge=10, boundary_K=25, sin_cos_deg=59, scale_factor=2,
                             inverse_deg=1),
    "bert_n65536_qkv": dict(log_n=16, bits=BERT_BITS, seed=seed8(600), hamming_weight=192, scale_log2=46,
                            weight_seed=11, token_seed=12, lane=0, proj_limbs=2),
}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


class SealKeys:
    """A seeded SEAL context whose Galois keys are made one element at a time
    (with one seed per factory, a key does not depend on which others exist)
    and kept in a small LRU, since 47 keys at N=2^16 do not fit in memory."""

    def __init__(self, log_n, qs, seed, hamming_weight, keep=10):
        self.ref = pr.SealRef(log_n, qs, seed=np.array(seed, dtype=np.uint64), hamming_weight=hamming_weight)
        self.cache = OrderedDict()
        self.keep = keep
        self.elts = set()
        self.made = 0

    def allow(self, elts):
        self.elts |= set(int(e) for e in elts)
        return self

    def __contains__(self, elt):
        return int(elt) in self.elts

    def __getitem__(self, elt):
        elt = int(elt)
        if elt not in self.elts:
            raise KeyError(elt)
        if elt in self.cache:
            self.cache.move_to_end(elt)
            return self.cache[elt]
        self.ref.galois_keys_from_elts([elt])
        k = self.ref.galois_key(elt)
        self.made += 1
        self.cache[elt] = k
        while len(self.cache) > self.keep:
            self.cache.popitem(last=False)
        return k

    def keys(self):
        return sorted(self.elts)


def case_keyswitch(c):
    n = 1 << c["log_n"]
    qs = po.create_coeff_modulus(n, c["bits"])
    ref = pr.SealRef(c["log_n"], qs, seed=np.array(c["seed"], dtype=np.uint64), hamming_weight=c["hamming_weight"])
    oc = po.OracleContext(c["log_n"], qs)
    l = c["limbs"]
    rng = np.random.default_rng(c["data_seed"])
    ct = po.random_residues(rng, (2, l, n), qs[:l])
    tgt = po.random_residues(rng, (1, l, n), qs[:l])[0]
    rk = ref.relin_key()
    out = {"relin_key": digest(rk), "switch_key": digest(oc.switch_key(ct, tgt, rk))}
    del rk
    elt = ref.galois_elt(c["rotate_step"])
    ref.galois_keys_from_elts([elt])
    gk = ref.galois_key(elt)
    out["galois_key"] = digest(gk)
    out["rotate"] = digest(oc.apply_galois(ct, elt, gk))
    return out


def case_gelu(c):
    n = 1 << c["log_n"]
    qs = po.create_coeff_modulus(n, c["bits"])
    ref = pr.SealRef(c["log_n"], qs, seed=np.array(c["seed"], dtype=np.uint64), hamming_weight=c["hamming_weight"])
    scale = 2.0 ** c["scale_log2"]
    oev = L.Evaluator(po.OracleContext(c["log_n"], qs), ref.relin_key(), {})
    ck = L.CKKSEvaluator(oev, scale)
    top = len(qs) - 1
    out = {}
    for inp in c["inputs"]:
        vals = np.random.default_rng(inp["data_seed"]).uniform(inp["lo"], inp["hi"], n // 2)
        pt = oev.encode(vals, scale, top).data
        ct = ref.encrypt_ntt(pt, scale, symmetric=True)
        res = L.gelu(ck, L.Ct(ct, scale))
        dec = ref.decrypt(res.data, res.scale)
        key = f"u{int(inp['lo'])}_{int(inp['hi'])}"
        out[key] = {"input": digest(ct), "output": digest(res.data), "scale": res.scale, "limbs": res.limbs,
                    "max_abs_err_vs_exact_gelu": float(np.max(np.abs(dec - _gelu(vals))))}
        print(f"  gelu {key}: limbs {res.limbs}", flush=True)
    return out


def _gelu(x):
    return 0.5 * x * (1.0 + np.tanh(math.sqrt(2.0 / math.pi) * (x + 0.044715 * x ** 3)))


def _partial_expand(omm, ct, leaves_needed):
    """expand_ciphertext (src/matrix_mul.cpp:101-129) computing only the nodes
    on the paths to `leaves_needed`: after level i, node a + b*2^i is the
    child (b = 0 left, 1 right) of node a, so leaf t's bit i is its choice at
    level i."""
    ev = omm.ev
    n = ev.n
    logn = int(round(math.log2(n)))
    nodes = {0: ct}
    for i in range(logn):
        keep = {t & ((2 << i) - 1) for t in leaves_needed}
        index_raw = (n << 1) - (1 << i)
        index = (index_raw * omm.rots[i]) % (n << 1)
        nxt = {}
        for a, node in nodes.items():
            want_l, want_r = a in keep, (a + (1 << i)) in keep
            if not (want_l or want_r):
                continue
            rotated = ev.apply_galois(node, omm.rots[i])
            if want_l:
                nxt[a] = ev.add(node, rotated)
            if want_r:
                nxt[a + (1 << i)] = ev.add(omm.multiply_power_of_x(node, index_raw),
                                           omm.multiply_power_of_x(rotated, index))
        nodes = nxt
    return nodes


def case_matmul(c):
    n = 1 << c["log_n"]
    qs = po.create_coeff_modulus(n, c["bits"])
    ref = pr.SealRef(c["log_n"], qs, seed=np.array(c["seed"], dtype=np.uint64), hamming_weight=c["hamming_weight"])
    rots = [(n + 2 ** i) // 2 ** i for i in range(c["log_n"])]
    ref.galois_keys_from_elts(rots)
    gks = {e: ref.galois_key(e) for e in rots}
    oev = L.Evaluator(po.OracleContext(c["log_n"], qs), None, gks)
    pt_scale = 2.0 ** c["pt_scale_log2"]
    omm = L.MMEvaluator(L.CKKSEvaluator(oev, pt_scale))
    rows, cols, outc = c["rows"], c["cols"], c["out"]
    rng = np.random.default_rng(c["data_seed"])
    X = rng.normal(0, 1, (rows, cols))
    W = rng.normal(0, 0.02, (cols, outc))
    b = rng.normal(0, 0.02, outc)
    flat = X.reshape(-1)
    packs = []
    for i in range((flat.size + n - 1) // n):
        chunk = np.zeros(n)
        part = flat[i * n:(i + 1) * n]
        chunk[:part.size] = part
        data, sc = ref.mm_compress(chunk, pt_scale)
        assert sc == c["pack_scale"]
        packs.append(L.Ct(data, sc))
    out = {"compressed": [digest(p.data) for p in packs], "rows": {}}
    pts = [L.Pt(pt_scale, data=oev.encode(W[k], pt_scale, 2).data) for k in range(cols)]
    for r in c["check_rows"]:
        t0 = time.time()
        e0, e1 = r * cols, (r + 1) * cols
        leaves = {}
        for ci in range(e0 // n, (e1 - 1) // n + 1):
            need = [e - ci * n for e in range(max(e0, ci * n), min(e1, (ci + 1) * n))]
            nodes = _partial_expand(omm, packs[ci], need)
            for t in need:
                leaves[ci * n + t] = nodes[t]
        acc = None
        for k in range(cols):
            term = oev.multiply_plain(leaves[e0 + k], pts[k])
            acc = term if acc is None else oev.add(acc, term)
        acc.scale *= float(n)
        while acc.limbs > 1:
            acc = oev.rescale(acc)
        acc = oev.add_plain(acc, oev.encode(b, acc.scale, acc.limbs))
        dec = ref.decrypt(acc.data, acc.scale)[:outc]
        out["rows"][str(r)] = {"output": digest(acc.data), "scale": acc.scale, "limbs": acc.limbs,
                               "max_abs_err_vs_fp64": float(np.max(np.abs(dec - (X[r] @ W + b))))}
        print(f"  matmul row {r}: {time.time() - t0:.0f} s", flush=True)
    return out


def case_bootstrap(c):
    from nexus_gb300.remez import load_table
    n = 1 << c["log_n"]
    log_nh = c["log_n"] - 1
    qs = po.create_coeff_modulus(n, c["bits"])
    keys = SealKeys(c["log_n"], qs, c["seed"], c["hamming_weight"])
    steps = B.rot_key_steps_3(log_nh, log_nh)
    keys.allow(keys.ref.galois_elt(s) for s in steps)
    scale = 2.0 ** c["scale_log2"]
    oev = L.Evaluator(po.OracleContext(c["log_n"], qs), keys.ref.relin_key(), keys)
    obs = B.Bootstrapper(oev, c["loge"], log_nh, log_nh, len(qs) - 2, scale, c["boundary_K"], c["sin_cos_deg"],
                         c["scale_factor"], c["inverse_deg"], load_table())
    obs.generate_LT_coefficient_3()
    top = len(qs) - 1
    vals = np.random.default_rng(c["data_seed"]).uniform(-1, 1, n // 2)
    pt = oev.encode(vals, scale, top).data
    ct = keys.ref.encrypt_ntt(pt, scale, symmetric=True)
    low = np.ascontiguousarray(ct[:, :1, :])
    out = {"input": digest(low)}
    t0 = time.time()
    ox = L.Ct(low, scale)
    obs.initial_scale = ox.scale
    raised = obs.modraise_inplace(ox)
    out["modraise"] = digest(raised.data)
    raised.scale = float(qs[0])
    r1, r2 = obs.coefftoslot_full_3(raised)
    out["coefftoslot"] = [digest(r1.data), digest(r2.data)]
    print(f"  bootstrap CoeffToSlot done ({time.time() - t0:.0f} s, {keys.made} keys made)", flush=True)
    m1 = obs.modular_reduction(r1)
    m2 = obs.modular_reduction(r2)
    out["modular_reduction"] = [digest(m1.data), digest(m2.data)]
    out["modular_reduction_scale"] = [m1.scale, m2.scale]
    res = obs.slottocoeff_full_3(m1, m2)
    res.scale = obs.final_scale
    out["output"] = digest(res.data)
    out["output_limbs"] = res.limbs
    out["output_scale"] = res.scale
    dec = keys.ref.decrypt(res.data, res.scale).real
    out["max_abs_err_vs_input"] = float(np.max(np.abs(dec - vals)))
    print(f"  bootstrap done ({time.time() - t0:.0f} s, {keys.made} keys made)", flush=True)
    return out


def case_bert_qkv(c):
    """The encrypted BERT-base layer's Q, K and V projections (block-diagonal
    BSGS transforms of the engine's BertLayerT, restated in oracle/bert.py) for
    the lane of the 128-token request, on the ciphertexts the layer receives:
    the packed tokens encrypted at the top level, switched down to two limbs."""
    from nexus_gb300 import bert as NB
    from oracle import bert as OB

    class _Scale:
        final_scale = 2.0 ** c["scale_log2"]

    n = 1 << c["log_n"]
    qs = po.create_coeff_modulus(n, c["bits"])
    sh = NB.BertShape()
    w = NB.random_weights(sh, np.random.default_rng(c["weight_seed"]))
    rng = np.random.default_rng(c["token_seed"])
    tokens = [[rng.normal(0, 1, (Lr, sh.hidden)) for (_, Lr) in lane] for lane in sh.lanes]
    osh = OB.Shape(n // 2, sh.hidden, sh.heads, sh.head_dim, sh.ffn, sh.T, sh.lanes, sh.boot_shrink)
    keys = SealKeys(c["log_n"], qs, c["seed"], c["hamming_weight"], keep=30)
    keys.allow(keys.ref.galois_elt(s) for s in osh.rotation_steps())
    scale = 2.0 ** c["scale_log2"]
    oev = L.Evaluator(po.OracleContext(c["log_n"], qs), keys.ref.relin_key(), keys)
    layer = OB.BertLayer(oev, _Scale(), osh, w, c["lane"])
    top = len(qs) - 1
    x, inputs = [], []
    for v in NB.pack_lane(sh, n // 2, c["lane"], tokens[c["lane"]]):
        ct = keys.ref.encrypt_ntt(oev.encode(v, scale, top).data, scale, symmetric=True)
        inputs.append(digest(ct))
        x.append(L.Ct(np.ascontiguousarray(ct[:, :c["proj_limbs"], :]), scale))
    out = {"input": inputs}
    t0 = time.time()
    for which, name in ((0, "q"), (1, "k"), (2, "v")):
        y = layer.project(x, which)
        out[name] = [digest(ct.data) for ct in y]
        out[name + "_scale"] = y[0].scale
        out[name + "_limbs"] = y[0].limbs
        print(f"  projection {name} done ({time.time() - t0:.0f} s, {keys.made} keys made)", flush=True)
    return out


RUN = {"keyswitch_n65536_l31": case_keyswitch, "gelu_n16384": case_gelu, "matmul_n65536": case_matmul,
       "bootstrap_n65536": case_bootstrap, "bert_n65536_qkv": case_bert_qkv}


def main(argv):
    assert pr.available(), "SEAL reference build unavailable"
    po.set_threads(os.cpu_count() or 1)
    doc = json.loads(OUT.read_text()) if OUT.exists() else {"cases": {}}
    for name in (argv or list(CASES)):
        c = CASES[name]
        t0 = time.time()
        print(name, flush=True)
        n = 1 << c["log_n"]
        rec = dict(c, moduli=[str(q) for q in po.create_coeff_modulus(n, c["bits"])])
        rec["sha256"] = RUN[name](c)
        rec["seconds"] = round(time.time() - t0, 1)
        doc["cases"][name] = rec
        OUT.write_text(json.dumps(doc, indent=1) + "\n")
        print(f"{name} done in {rec['seconds']} s", flush=True)


if __name__ == "__main__":
    main(sys.argv[1:])
