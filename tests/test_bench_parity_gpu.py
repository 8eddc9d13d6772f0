"""Word parity at the configurations bench.py measures, from seeds alone.

tests/golden/bench_digests.json (made by tests/golden/make_bench_digests.py
with the real SEAL-4.1-bs for keys and encryptions and the oracle for the
evaluation) holds SHA-256 digests of the output words of: a key switch and a
rotation at 31 limbs on the N=2^16 bootstrap chain, GELU at N=2^14 on the
reference chain (inputs U(-5,5) and U(-8,8)), three rows of the BERT-shape
MatMul at N=2^16 and every stage of a full-slot bootstrap at N=2^16 with
h = 192.  Here the engine makes the same keys and encryptions on the GPU
from the same seeds (nexus_seal_*), runs the same operations -- single and
lockstep forms -- and must reproduce every digest."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from tests.util import to_dev, to_host

pytestmark = pytest.mark.gpu

DOC = json.loads((Path(__file__).parent / "golden" / "bench_digests.json").read_text())["cases"]


def _digest(t) -> str:
    """SHA-256 of the little-endian words, one leading-axis slice at a time."""
    h = hashlib.sha256()
    a = t if isinstance(t, np.ndarray) else None
    if a is not None:
        h.update(np.ascontiguousarray(a, dtype="<u8").tobytes())
        return h.hexdigest()
    for part in t.reshape(t.shape[0], -1):
        h.update(to_host(part).astype("<u8").tobytes())
    return h.hexdigest()


def _ctx(c):
    import nexus_gb300 as ng
    qs = [int(q) for q in c["moduli"]]
    assert qs == ng.create_coeff_modulus(1 << c["log_n"], c["bits"])
    return ng.Context(c["log_n"], qs), qs


def _seed(c):
    return np.array(c["seed"], dtype=np.uint64)


def test_keyswitch_l31(cuda):
    import torch
    from oracle import pyoracle as po
    c = DOC["keyswitch_n65536_l31"]
    d = c["sha256"]
    ctx, qs = _ctx(c)
    n, l = 1 << c["log_n"], c["limbs"]
    sk = ctx.seal_keygen_secret(_seed(c), c["hamming_weight"])
    rk = ctx.seal_keygen_relin(sk, _seed(c))
    assert _digest(rk) == d["relin_key"]
    rng = np.random.default_rng(c["data_seed"])
    ct = po.random_residues(rng, (2, l, n), qs[:l])
    tgt = po.random_residues(rng, (1, l, n), qs[:l])[0]
    dct = to_dev(ct)
    ctx.switch_key(dct, to_dev(tgt), rk)
    assert _digest(dct) == d["switch_key"]
    del rk
    elt = ctx.galois_elt(c["rotate_step"])
    gk = ctx.seal_keygen_galois(sk, elt, _seed(c))
    assert _digest(gk) == d["galois_key"]
    out = torch.empty_like(dct)
    ctx.apply_galois(to_dev(ct), elt, gk, out)
    assert _digest(out) == d["rotate"]


def test_gelu_n16384(cuda):
    import torch
    from nexus_gb300.operators import Ciphertext, Evaluator
    c = DOC["gelu_n16384"]
    ctx, qs = _ctx(c)
    n = 1 << c["log_n"]
    scale = 2.0 ** c["scale_log2"]
    sk = ctx.seal_keygen_secret(_seed(c), c["hamming_weight"])
    rk = ctx.seal_keygen_relin(sk, _seed(c))
    ev = Evaluator(ctx, scale, rk)
    top = len(qs) - 1
    cts, wants = [], []
    for inp in c["inputs"]:
        want = c["sha256"][f"u{int(inp['lo'])}_{int(inp['hi'])}"]
        vals = np.random.default_rng(inp["data_seed"]).uniform(inp["lo"], inp["hi"], n // 2)
        pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
        ctx.encode(vals, scale, top, pt)
        ct = ctx.seal_encrypt_symmetric(sk, pt, top, _seed(c))
        assert _digest(ct) == want["input"]
        cts.append(ct)
        wants.append(want)
    single = [ev.gelu(Ciphertext.from_device(ctx, ct, scale)) for ct in cts]
    batch = ev.gelu_batch([Ciphertext.from_device(ctx, ct, scale) for ct in cts])
    for got, lock, want in zip(single, batch, wants):
        assert got.scale == want["scale"] and got.to_numpy().shape[1] == want["limbs"]
        assert _digest(got.to_numpy()) == want["output"]
        assert _digest(lock.to_numpy()) == want["output"]


def test_matmul_bert_rows(cuda):
    import torch
    from nexus_gb300.operators import Ciphertext, Evaluator
    c = DOC["matmul_n65536"]
    d = c["sha256"]
    ctx, qs = _ctx(c)
    n = 1 << c["log_n"]
    pt_scale = 2.0 ** c["pt_scale_log2"]
    sk = ctx.seal_keygen_secret(_seed(c), c["hamming_weight"])
    pk = ctx.seal_keygen_public(sk, _seed(c))
    rots = [(n + 2 ** i) // 2 ** i for i in range(c["log_n"])]
    gks = {e: ctx.seal_keygen_galois(sk, e, _seed(c)) for e in rots}
    ev = Evaluator(ctx, pt_scale, None, gks)
    rows, cols, outc = c["rows"], c["cols"], c["out"]
    rng = np.random.default_rng(c["data_seed"])
    X = rng.normal(0, 1, (rows, cols))
    W = rng.normal(0, 0.02, (cols, outc))
    b = rng.normal(0, 0.02, outc)
    flat = X.reshape(-1)
    packs = []
    for i in range((flat.size + n - 1) // n):
        # enc_compress_ciphertext: a public-key encryption of zero plus the
        # coefficient-packed values at scale 1e10
        ct = ctx.seal_encrypt(pk, None, 2, _seed(c))
        pt = torch.empty((2, n), dtype=torch.int64, device="cuda")
        ctx.encode_coefficients(flat[i * n:(i + 1) * n], c["pack_scale"], 2, pt)
        c0 = ct[0:1].clone()
        ctx.plain_op(c0, pt, 1, ct[0:1])
        assert _digest(ct) == d["compressed"][i]
        packs.append(Ciphertext.from_device(ctx, ct, c["pack_scale"]))
    pts = torch.empty((cols, 2, n), dtype=torch.int64, device="cuda")
    for k in range(cols):
        ctx.encode(W[k], pt_scale, 2, pts[k])
    res = ev.matrix_mul(packs, pts, pt_scale, rows, cols, float(n), bias=b)
    for r in c["check_rows"]:
        want = d["rows"][str(r)]
        assert res[r].scale == want["scale"]
        assert _digest(res[r].to_numpy()) == want["output"], r


def test_bootstrap_n65536_stages(cuda):
    import torch
    from nexus_gb300.operators import (BOOT_COEFFTOSLOT, BOOT_MODRAISE, BOOT_MODULAR_REDUCTION,
                                       BOOT_SET_INITIAL_SCALE, BOOT_SLOTTOCOEFF, Bootstrapper, Ciphertext,
                                       Evaluator)
    c = DOC["bootstrap_n65536"]
    d = c["sha256"]
    ctx, qs = _ctx(c)
    n = 1 << c["log_n"]
    log_nh = c["log_n"] - 1
    scale = 2.0 ** c["scale_log2"]
    sk = ctx.seal_keygen_secret(_seed(c), c["hamming_weight"])
    rk = ctx.seal_keygen_relin(sk, _seed(c))
    ev = Evaluator(ctx, scale, rk)
    bs = Bootstrapper(ev, c["loge"], log_nh, log_nh, len(qs) - 2, scale, c["boundary_K"], c["sin_cos_deg"],
                      c["scale_factor"], c["inverse_deg"])
    for st in bs.rotation_steps(log_nh):
        e = ctx.galois_elt(st)
        ev.add_galois_key(e, ctx.seal_keygen_galois(sk, e, _seed(c)))
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    top = len(qs) - 1
    vals = np.random.default_rng(c["data_seed"]).uniform(-1, 1, n // 2)
    pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
    ctx.encode(vals, scale, top, pt)
    low = ctx.seal_encrypt_symmetric(sk, pt, top, _seed(c))[:, :1, :].contiguous()
    assert _digest(low) == d["input"]
    host_low = to_host(low).copy()

    # stage by stage
    x = Ciphertext.from_numpy(ctx, host_low, scale)
    bs.stage(BOOT_SET_INITIAL_SCALE, x)
    bs.stage(BOOT_MODRAISE, x)
    assert _digest(x.to_numpy()) == d["modraise"]
    x = Ciphertext.from_numpy(ctx, x.to_numpy(), float(qs[0]))
    r1, r2 = bs.stage(BOOT_COEFFTOSLOT, x)
    assert [_digest(r1.to_numpy()), _digest(r2.to_numpy())] == d["coefftoslot"]
    m1, _ = bs.stage(BOOT_MODULAR_REDUCTION, r1)
    m2, _ = bs.stage(BOOT_MODULAR_REDUCTION, r2)
    assert [_digest(m1.to_numpy()), _digest(m2.to_numpy())] == d["modular_reduction"]
    assert [m1.scale, m2.scale] == d["modular_reduction_scale"]
    out, _ = bs.stage(BOOT_SLOTTOCOEFF, m1, m2)
    assert _digest(out.to_numpy()) == d["output"]

    # whole bootstrap_3, and the lockstep form with a second ciphertext
    whole = bs.bootstrap_3(Ciphertext.from_numpy(ctx, host_low, scale))
    assert whole.scale == d["output_scale"] and whole.to_numpy().shape[1] == d["output_limbs"]
    assert _digest(whole.to_numpy()) == d["output"]
    other = Ciphertext.from_numpy(ctx, host_low[:, :, ::-1].copy(), scale)
    batch = bs.bootstrap_batch([Ciphertext.from_numpy(ctx, host_low, scale), other])
    assert _digest(batch[0].to_numpy()) == d["output"]
    dec = ctx.decode(ctx.decrypt(sk, whole.to_device()), whole.scale).real
    assert np.max(np.abs(dec - vals)) < 2.0 ** -10


def test_bert_qkv_projections(cuda):
    """The BERT-base layer's Q, K and V projections for the 128-token lane at
    N=2^16, on the inputs bench.py's layer receives (SEAL keys and
    encryptions from seed 600, weights and tokens from seeds 11 and 12)."""
    import torch
    from nexus_gb300 import bert as NB
    from nexus_gb300.operators import Bootstrapper, Ciphertext, Evaluator
    if "bert_n65536_qkv" not in DOC:
        pytest.skip("no digests for the BERT projections")
    c = DOC["bert_n65536_qkv"]
    d = c["sha256"]
    ctx, qs = _ctx(c)
    n = 1 << c["log_n"]
    scale = 2.0 ** c["scale_log2"]
    sk = ctx.seal_keygen_secret(_seed(c), c["hamming_weight"])
    ev = Evaluator(ctx, scale, ctx.seal_keygen_relin(sk, _seed(c)))
    log_nh = c["log_n"] - 1
    bs = Bootstrapper(ev, 10, log_nh, log_nh, len(qs) - 2, scale, 25, 59, 2, 1)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    sh = NB.BertShape()
    w = NB.random_weights(sh, np.random.default_rng(c["weight_seed"]))
    rng = np.random.default_rng(c["token_seed"])
    tokens = [[rng.normal(0, 1, (L, sh.hidden)) for (_, L) in lane] for lane in sh.lanes]
    layer = NB.BertLayer(bs, sh, w)
    for st in layer.rotation_steps():
        e = ctx.galois_elt(st)
        ev.add_galois_key(e, ctx.seal_keygen_galois(sk, e, _seed(c)))
    top = len(qs) - 1
    pl = c["proj_limbs"]
    x = []
    for lane in range(len(sh.lanes)):
        for i, v in enumerate(NB.pack_lane(sh, n // 2, lane, tokens[lane])):
            pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
            ctx.encode(v, scale, top, pt)
            ct = ctx.seal_encrypt_symmetric(sk, pt, top, _seed(c))
            if lane == c["lane"]:
                assert _digest(ct) == d["input"][i]
            x.append(Ciphertext.from_device(ctx, ct[:, :pl, :].contiguous(), scale))
            del pt, ct
    nh = layer.n_head
    for which, name in ((0, "q"), (1, "k"), (2, "v")):
        for lockstep in (True, False):
            y = layer.stage(NB.BERT_PROJECT, which, x, nh, lockstep)
            lane_y = y[c["lane"] * nh:(c["lane"] + 1) * nh]
            assert lane_y[0].scale == d[name + "_scale"]
            assert lane_y[0].to_numpy().shape[1] == d[name + "_limbs"]
            assert [_digest(t.to_numpy()) for t in lane_y] == d[name], (name, lockstep)
