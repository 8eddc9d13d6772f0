"""Encrypted BERT encoder layer on the GPU against the oracle (oracle/bert.py),
word for word, at the reduced size of tests/golden/bert_digests.json (N = 2^13,
128 token slots per block, hidden 64, 2 heads, FFN 160, requests of 40 | 8 + 32
tokens in two lanes): the Q/K/V projections, their bootstrap, the attention
block and the whole layer in its single-lane and lockstep forms (two
ciphertexts per bootstrap and the FFN fold, the defaults), with keys and
encryptions made from the same SEAL seed; plus the decrypted output against
the FP64 layer with NEXUS's approximations, with and without the packing."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

from tests.util import to_host

pytestmark = pytest.mark.gpu

DOC = json.loads((Path(__file__).parent / "golden" / "bert_digests.json").read_text())


def _digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def _shape():
    from nexus_gb300 import bert as NB
    c = DOC
    return NB.BertShape(hidden=c["hidden"], heads=c["heads"], head_dim=c["head_dim"], ffn=c["ffn"], T=c["T"],
                        lanes=[[tuple(r) for r in lane] for lane in c["lanes"]], boot_shrink=c["boot_shrink"],
                        boot_pack=c["boot_pack"], token_fold=c["token_fold"])


@pytest.fixture(scope="module")
def env(cuda):
    import torch
    import nexus_gb300 as ng
    from nexus_gb300 import bert as NB
    from nexus_gb300.operators import Bootstrapper, Ciphertext, Evaluator
    c = DOC
    n = 1 << c["log_n"]
    qs = [int(q) for q in c["moduli"]]
    assert qs == ng.create_coeff_modulus(n, c["bits"])
    ctx = ng.Context(c["log_n"], qs)
    seed = np.array(c["seed"], dtype=np.uint64)
    scale = 2.0 ** c["scale_log2"]
    sk = ctx.seal_keygen_secret(seed, c["hamming_weight"])
    ev = Evaluator(ctx, scale, ctx.seal_keygen_relin(sk, seed))
    log_nh = c["log_n"] - 1
    bs = Bootstrapper(ev, c["loge"], log_nh, log_nh, len(qs) - 2, scale, c["boundary_K"], c["sin_cos_deg"],
                      c["scale_factor"], c["inverse_deg"])
    sh = _shape()
    w = NB.random_weights(sh, np.random.default_rng(c["weight_seed"]))
    rng = np.random.default_rng(c["token_seed"])
    tokens = [[rng.normal(0, 1, (L, sh.hidden)) for (_, L) in lane] for lane in sh.lanes]
    steps = bs.rotation_steps(log_nh)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    layer = NB.BertLayer(bs, sh, w)
    assert layer.rotation_steps() == c["rotation_steps"]
    for s in steps + [s for s in layer.rotation_steps() if s not in steps]:
        e = ctx.galois_elt(s)
        ev.add_galois_key(e, ctx.seal_keygen_galois(sk, e, seed))
    top = len(qs) - 1
    x = []
    for lane in range(len(sh.lanes)):
        for i, v in enumerate(NB.pack_lane(sh, n // 2, lane, tokens[lane])):
            pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
            ctx.encode(v, scale, top, pt)
            ct = ctx.seal_encrypt_symmetric(sk, pt, top, seed)
            assert _digest(to_host(ct)) == c["lanes_out"][lane]["input"][i]
            x.append(Ciphertext.from_device(ctx, ct, scale))
    return dict(ctx=ctx, sk=sk, ev=ev, bs=bs, layer=layer, sh=sh, w=w, tokens=tokens, x=x, n=n)


def _lane_digests(cts, per_lane):
    return [[_digest(c.to_numpy()) for c in cts[l * per_lane:(l + 1) * per_lane]]
            for l in range(len(cts) // per_lane)]


def _want(stage):
    return [lane["stages"][stage] for lane in DOC["lanes_out"]]


def _truncate(ctx, cts, limbs):
    from nexus_gb300.operators import Ciphertext
    return [Ciphertext.from_numpy(ctx, c.to_numpy()[:, :limbs, :].copy(), c.scale) for c in cts]


@pytest.mark.parametrize("lockstep", [False, True])
def test_qkv_and_attention_stages(env, lockstep):
    """The forward's first blocks stage by stage: Q and K on the lower half of
    each token block, V; Q and K folded two per ciphertext (token fold),
    refreshed together, Q unfolded at the attention's level (14 limbs) and K
    one level above it with its second token copies rebuilt; the attention."""
    from nexus_gb300.bert import (BERT_ATTENTION, BERT_BOOTSTRAP, BERT_FOLD, BERT_LOWER_HALF, BERT_PROJECT,
                                  BERT_UNFOLD)
    layer, ctx = env["layer"], env["ctx"]
    nl, nh = layer.n_lanes, layer.n_head
    assert DOC["token_fold"] and nh == 2
    nq = (nh + 1) // 2
    # Q and K from the input at 2 limbs, V at 4 (it lands at the attention's level unrefreshed)
    x2, x4 = _truncate(ctx, env["x"], 2), _truncate(ctx, env["x"], 4)
    proj = [layer.stage(BERT_PROJECT, w, x, nh, lockstep)
            for w, x in ((0 | BERT_LOWER_HALF, x2), (1 | BERT_LOWER_HALF, x2), (2, x4))]
    # lane-major q | k | v per lane
    qkv = [proj[t][l * nh + i] for l in range(nl) for t in range(3) for i in range(nh)]
    assert _lane_digests(qkv, 3 * nh) == _want("qkv")
    qf, kf = (layer.stage(BERT_FOLD, 0, proj[t], nq, lockstep) for t in (0, 1))
    qk = [c for l in range(nl) for c in qf[l * nq:(l + 1) * nq] + kf[l * nq:(l + 1) * nq]]
    boot = layer.stage(BERT_BOOTSTRAP, 0, qk, 2 * nq, lockstep)
    assert _lane_digests(boot, 2 * nq) == _want("qk_boot")
    q14 = _truncate(ctx, [boot[l * 2 * nq + i] for l in range(nl) for i in range(nq)], 14)
    k15 = _truncate(ctx, [boot[l * 2 * nq + nq + i] for l in range(nl) for i in range(nq)], 15)
    q = layer.stage(BERT_UNFOLD, 0, q14, nh, lockstep)
    k = layer.stage(BERT_UNFOLD, 1, k15, nh, lockstep)
    att_in = [c for l in range(nl) for c in q[l * nh:(l + 1) * nh] + k[l * nh:(l + 1) * nh]
              + proj[2][l * nh:(l + 1) * nh]]
    assert _lane_digests(att_in, 3 * nh) == _want("qkv_boot")
    att = layer.stage(BERT_ATTENTION, 0, att_in, nh, lockstep)
    assert _lane_digests(att, nh) == _want("attention")


def test_fold_stages_reject_wrong_counts(env):
    from nexus_gb300 import NexusError
    from nexus_gb300.bert import BERT_FOLD, BERT_UNFOLD
    layer = env["layer"]
    x = env["x"]                                  # 2 per lane
    with pytest.raises(NexusError, match="count"):
        layer.stage(BERT_FOLD, 0, x, 2, True)      # 2 -> 1, not 2
    with pytest.raises(NexusError, match="count"):
        layer.stage(BERT_UNFOLD, 0, x, 2, True)    # 2 unfold to 3 or 4, not 2


@pytest.mark.parametrize("lockstep", [False, True])
def test_layer_matches_oracle(env, lockstep):
    from nexus_gb300 import bert as NB
    layer, ctx, sh, n = env["layer"], env["ctx"], env["sh"], env["n"]
    out = layer.forward(env["x"], lockstep)
    got = _lane_digests(out, layer.n_hid)
    assert got == _want("output")
    for lane in range(layer.n_lanes):
        cts = out[lane * layer.n_hid:(lane + 1) * layer.n_hid]
        assert cts[0].scale == DOC["lanes_out"][lane]["output_scale"]
        dec = np.stack([ctx.decode(ctx.decrypt(env["sk"], c.to_device()), c.scale).real for c in cts])
        ys = NB.unpack_lane(sh, n // 2, lane, dec)
        ref = NB.layer_reference(sh, env["w"], env["tokens"][lane])
        err = max(float(np.max(np.abs(y - r))) for y, r in zip(ys, ref))
        assert err < 2.0 ** -7, err


@pytest.mark.parametrize("pack,fold", [(False, False), (True, False), (False, True)])
def test_other_packings_keep_the_layer_within_its_error(env, pack, fold):
    """With one ciphertext per bootstrap (boot_pack off), the FFN unfolded
    (token_fold off), or both (the plain form), the layer's lockstep and
    single-lane forms agree word for word, and the decrypted output stays
    within the default layer's error bound against the FP64 layer."""
    from nexus_gb300 import bert as NB
    layer, ctx, sh, n = env["layer"], env["ctx"], env["sh"], env["n"]
    layer.set_boot_pack(pack)
    layer.set_token_fold(fold)
    try:
        lock = layer.forward(env["x"], True)
        single = layer.forward(env["x"], False)
    finally:
        layer.set_boot_pack(True)
        layer.set_token_fold(True)
    for a, b in zip(lock, single):
        assert np.array_equal(a.to_numpy(), b.to_numpy())
    for lane in range(layer.n_lanes):
        cts = lock[lane * layer.n_hid:(lane + 1) * layer.n_hid]
        dec = np.stack([ctx.decode(ctx.decrypt(env["sk"], c.to_device()), c.scale).real for c in cts])
        ys = NB.unpack_lane(sh, n // 2, lane, dec)
        ref = NB.layer_reference(sh, env["w"], env["tokens"][lane])
        err = max(float(np.max(np.abs(y - r))) for y, r in zip(ys, ref))
        assert err < 2.0 ** -7, err
