"""Host-side pieces of the encrypted BERT layer (no GPU): the client packing
round trip, the FP64 reference's NEXUS approximations against the exact
functions on their domains, the oracle's packing restatement against the
engine package's, and argument rejection of the layer's C ABI."""
import ctypes

import numpy as np

from nexus_gb300 import bert as NB


def _small_shape():
    return NB.BertShape(hidden=64, heads=2, head_dim=32, ffn=128, T=32, lanes=[[(0, 16)], [(0, 4), (8, 8)]])


def test_pack_unpack_round_trip():
    sh = _small_shape()
    slots = 4096
    rng = np.random.default_rng(0)
    for lane, reqs in enumerate(sh.lanes):
        toks = [rng.normal(size=(L, sh.hidden)) for (_, L) in reqs]
        vecs = NB.pack_lane(sh, slots, lane, toks)
        assert vecs.shape == (sh.n_hid(slots), slots)
        back = NB.unpack_lane(sh, slots, lane, vecs)
        for a, b in zip(toks, back):
            assert np.array_equal(a, b)
        # the second token copy holds the same values
        for (o, L), x in zip(reqs, toks):
            for f in (0, sh.hidden - 1):
                c, j = divmod(f, slots // sh.T)
                assert np.array_equal(vecs[c, j * sh.T + o + L:j * sh.T + o + 2 * L], x[:, f])


def test_nexus_approximations_on_their_domains():
    x = np.linspace(-2.0, 0.0, 50)
    assert np.max(np.abs(NB.nexus_exp(x) - np.exp(x))) < 2e-2
    y = np.linspace(0.2, 1.8, 50)
    assert np.max(np.abs(NB.nexus_inverse(y) - 1.0 / y) / (1.0 / y)) < 0.2
    z = np.linspace(5.0, 500.0, 50)
    assert np.max(np.abs(NB.nexus_invert_sqrt(z) - 1.0 / np.sqrt(z)) * np.sqrt(z)) < 1e-2
    g = np.linspace(-4.0, 4.0, 81)
    exact = 0.5 * g * (1.0 + np.tanh(np.sqrt(2.0 / np.pi) * (g + 0.044715 * g ** 3)))
    assert np.max(np.abs(NB.nexus_gelu(g) - exact)) < 2e-2


def test_layer_reference_shapes_and_exact_softmax_rows():
    sh = _small_shape()
    w = NB.random_weights(sh, np.random.default_rng(1))
    toks = [np.random.default_rng(2).normal(size=(6, sh.hidden))]
    approx = NB.layer_reference(sh, w, toks)
    exact = NB.layer_reference(sh, w, toks, exact=True)
    assert approx[0].shape == exact[0].shape == (6, sh.hidden)
    assert np.all(np.isfinite(approx[0]))
    # the exact layer's outputs are LayerNorm'd: unit mean square per token
    assert np.allclose(np.mean(exact[0] ** 2, axis=1), 1.0)


def test_oracle_restates_the_rotation_steps():
    from oracle import bert as OB
    sh = _small_shape()
    osh = OB.Shape(4096, sh.hidden, sh.heads, sh.head_dim, sh.ffn, sh.T, sh.lanes, sh.boot_shrink)
    steps = osh.rotation_steps()
    assert len(steps) == len(set(steps)) and all(0 < s < 4096 for s in steps)
    # baby steps of the block transforms, the attention's token shifts, the folds
    assert sh.T in steps and 1 in steps and (osh.H2 * sh.T) in steps


def test_layer_abi_rejects_null_arguments_without_gpu():
    from nexus_gb300 import _lib
    lib = _lib.lib()
    out = ctypes.c_void_p()
    one = (ctypes.c_int * 1)(1)
    req = (ctypes.c_int * 2)(0, 4)
    assert lib.nexus_bert_layer_create(None, 64, 2, 32, 128, 32, 1, one, req, ctypes.c_double(2.0), None,
                                       ctypes.byref(out)) != 0
    assert lib.nexus_last_error().startswith(b"nexus_bert_layer_create") and b"null" in lib.nexus_last_error()
    assert lib.nexus_bert_layer_forward(None, 1, None, None) != 0
    assert lib.nexus_bert_layer_stage(None, 1, 0, 0, None, 0, None, 0) != 0
    n = ctypes.c_int()
    assert lib.nexus_bert_layer_rotation_steps(None, None, ctypes.byref(n), 0) != 0


class _Slots:
    """A plaintext stand-in for the oracle's ciphertexts: slot values only."""

    def __init__(self, v, limbs=3, scale=1.0):
        self.v, self.limbs, self.scale = np.asarray(v, dtype=float), limbs, scale


class _SlotEvaluator:
    """The oracle evaluator's interface over slot vectors: rotate(x, k) moves
    slot i + k to slot i (CKKS rotate_vector), rescale drops a limb."""

    q = [2.0 ** 40] * 8

    def rotate(self, x, k):
        return _Slots(np.roll(x.v, -k), x.limbs, x.scale)

    def add(self, a, b):
        return _Slots(a.v + b.v, a.limbs, a.scale)

    def add_plain(self, a, p):
        return _Slots(a.v + p, a.limbs, a.scale)

    def multiply_plain(self, a, p):
        return _Slots(a.v * p, a.limbs, a.scale)

    def encode(self, v, scale, limbs):
        return np.asarray(v, dtype=float)

    def rescale(self, a):
        return _Slots(a.v, a.limbs - 1, a.scale)


def test_token_fold_slot_algebra():
    """The fold of BertLayerT (restated in oracle/bert.py): FFN1 on the lower
    half, h_2i + rot(h_2i+1, -T/2), an element-wise function, the unfold
    (2i+1 = rot(folded, T/2)) and FFN2 give the unfolded FFN's values on every
    lower-half token slot, which hold the numpy FFN of each token."""
    from oracle import bert as OB
    S, T, hidden, ffn = 256, 16, 16, 40
    lanes = [[(0, 4)], [(0, 2), (4, 3)]]
    osh = OB.Shape(S, hidden, 2, 8, ffn, T, lanes, 1.0)
    assert osh.fold_ok and osh.n_ffn == 3 and osh.n_hid == 1
    assert (T // 2) in osh.rotation_steps() and (S - T // 2) in osh.rotation_steps()
    rng = np.random.default_rng(5)
    w = {k: rng.normal(0, 0.5, s) for k, s in (("w1", (hidden, ffn)), ("w2", (ffn, hidden)), ("b1", ffn),
                                                ("b2", hidden))}
    layer = OB.BertLayer.__new__(OB.BertLayer)
    layer.ev, layer.sh, layer.w, layer.delta = _SlotEvaluator(), osh, w, 1.0
    X = rng.normal(size=(T, hidden))              # token slot t of every block holds token t
    x = [_Slots(np.concatenate([X[:, c * osh.NB + j] if c * osh.NB + j < hidden else np.zeros(T)
                                for j in range(osh.NB)])) for c in range(osh.n_hid)]

    def act(cts):
        return [_Slots(np.tanh(c.v), c.limbs, c.scale) for c in cts]

    plain = layer.project(act(layer.project(x, OB.LT_1)), OB.LT_2)
    folded_h = layer.fold_halves(layer.project(x, OB.LT_1, lower_half=True))
    assert len(folded_h) == 2
    folded = layer.project(layer.unfold_halves(act(folded_h), osh.n_ffn), OB.LT_2)
    want = np.tanh(X @ w["w1"] + w["b1"]) @ w["w2"] + w["b2"]          # [T][hidden]
    for c in range(osh.n_hid):
        for j in range(osh.NB):
            f = c * osh.NB + j
            if f >= hidden:
                continue
            blk = slice(j * T, (j + 1) * T)
            assert np.allclose(plain[c].v[blk], want[:, f])
            assert np.allclose(folded[c].v[blk][:T // 2], want[:T // 2, f])
    # requests reaching into the upper half turn the fold off
    assert not OB.Shape(S, hidden, 2, 8, ffn, T, [[(0, 9)]], 1.0).fold_ok


def test_unfold_copies_rebuilds_the_second_token_copies():
    """K's unfold (BertLayerT::unfold_copies, restated in oracle/bert.py):
    three ciphertexts written on the lower half of each token block, folded
    two per ciphertext, come back with every request's tokens and both token
    copies, including the copies that reach the upper half (rebuilt by one
    masked rotation per request length)."""
    from oracle import bert as OB
    S, T = 256, 32
    lanes = [[(0, 10)], [(0, 2), (4, 7)]]           # copies reaching slot 16 and up: lengths 10 and 7
    osh = OB.Shape(S, 16, 2, 8, 40, T, lanes, 1.0)
    assert osh.fold_ok and osh.copy_shifts == [7, 10]
    assert all((S - s) in osh.rotation_steps() for s in (7, 10, T // 2))
    rng = np.random.default_rng(9)
    for lane, reqs in enumerate(lanes):
        layer = OB.BertLayer.__new__(OB.BertLayer)
        layer.ev, layer.sh, layer.lane = _SlotEvaluator(), osh, lane
        full = []
        for _ in range(3):
            v = np.zeros(S)
            for j in range(S // T):
                for (o, L) in reqs:
                    tok = rng.normal(size=L)
                    v[j * T + o:j * T + o + L] = tok
                    v[j * T + o + L:j * T + o + 2 * L] = tok
            full.append(v)
        lower = [_Slots(np.where(np.arange(S) % T < T // 2, v, 0.0)) for v in full]
        out = layer.unfold_copies(layer.fold_halves(lower), 3)
        assert len(out) == 3 and out[0].limbs == lower[0].limbs - 1
        for got, want in zip(out, full):
            for j in range(S // T):
                for (o, L) in reqs:
                    sl = slice(j * T + o, j * T + o + 2 * L)
                    assert np.allclose(got.v[sl], want[sl])


def test_bench_bootstrap_count_follows_the_layer_shape():
    """bench.py's bootstraps per layer (the CPU lower bound's multiplier) is the
    count the layer's shape gives: per lane, Q and K folded two per ciphertext
    and refreshed in pairs, the row sum alone, each folded residual and the
    folded FFN hidden activations in pairs (an odd one alone)."""
    import bench
    from oracle import bert as OB

    def pairs(n):
        return (n + 1) // 2
    sh = NB.BertShape()                       # BERT-base, 128 | 32 + 64 tokens
    slots = 1 << 15
    osh = OB.Shape(slots, sh.hidden, sh.heads, sh.head_dim, sh.ffn, sh.T, sh.lanes, sh.boot_shrink)
    assert osh.folding and (osh.n_head, osh.n_hid, osh.n_ffn) == (8, 6, 24)
    for pack in (True, False):
        for fold in (True, False):
            f = pairs if fold else (lambda n: n)
            refresh = pairs if pack else (lambda n: n)
            per_lane = (refresh(2 * f(osh.n_head)) + 1 + 2 * refresh(f(osh.n_hid)) + refresh(f(osh.n_ffn)))
            assert bench.bert_bootstraps(pack, fold) == len(sh.lanes) * per_lane, (pack, fold)


class _Enc:
    """A stand-in ciphertext that keeps CKKS's encoded slot values m (the
    decoded value is m / scale), so that scale bookkeeping (rescale by the
    dropped prime, a scale reinterpreted by hand) means what it does on real
    ciphertexts."""

    def __init__(self, m, limbs, scale):
        self.m, self.limbs, self.scale = np.asarray(m, dtype=float), limbs, scale

    def value(self):
        return self.m / self.scale


class _EncPlain:
    def __init__(self, m, scale):
        self.m, self.scale = m, scale


class _EncEvaluator:
    """The oracle evaluator's interface on _Enc values (exact arithmetic on
    the encoded slot values, no noise)."""

    q = [float(2 ** 40 + 2 * i + 1) for i in range(32)]

    def rotate(self, x, k):
        return _Enc(np.roll(x.m, -k), x.limbs, x.scale)

    def add(self, a, b):
        assert np.isclose(a.scale, b.scale, rtol=1e-9)
        return _Enc(a.m + b.m, a.limbs, a.scale)

    def multiply(self, a, b):
        return _Enc(a.m * b.m, min(a.limbs, b.limbs), a.scale * b.scale)

    def relinearize(self, x):
        return x

    def square(self, x):
        return self.multiply(x, x)

    def rescale(self, x):
        qd = self.q[x.limbs - 1]
        return _Enc(x.m / qd, x.limbs - 1, x.scale / qd)

    def mod_switch_to(self, x, limbs):
        return _Enc(x.m, limbs, x.scale)

    def encode(self, v, scale, limbs):
        return _EncPlain(np.asarray(v, dtype=float) * scale, scale)

    def encode_scalar(self, value, scale, limbs):
        return _EncPlain(value * scale, scale)

    def multiply_plain(self, a, p):
        return _Enc(a.m * p.m, a.limbs, a.scale * p.scale)

    def add_plain(self, a, p):
        assert np.isclose(a.scale, p.scale, rtol=1e-9)
        return _Enc(a.m + p.m, a.limbs, a.scale)


class _EncCkks:
    """NEXUS's exp and inverse on decoded values (the oracle's CKKSEvaluator
    restates their ciphertext sequences; here only the layer's use of them
    is under test)."""

    def exp(self, x):
        return _Enc(NB.nexus_exp(x.value()) * x.scale, x.limbs - 8, x.scale)

    def inverse(self, x):
        return _Enc(NB.nexus_inverse(x.value()) * x.scale, x.limbs - 8, x.scale)

    def invert_sqrt(self, x, d_newt, d_gold):
        return _Enc(NB.nexus_invert_sqrt(x.value(), d_newt, d_gold) * x.scale, x.limbs - 17, x.scale)


def test_attention_fold_slot_algebra():
    """The oracle's attention block (BertLayerT::attention) on exact encoded
    slot values, with the token fold on and off: scores of offsets 2p and
    2p+1 folded after their zeroing mask, the head block sums per folded
    pair, the folded -128 masks, the row sums that add the other half of
    their own block (and take the 0.01 / 2 constant with the scale
    reinterpreted), P unfolded for the values.  Both give, on every first
    token copy, NEXUS's softmax attention of each request computed in numpy."""
    from oracle import bert as OB
    S, T, heads, dh = 512, 32, 2, 16
    lanes = [[(0, 6)], [(0, 3), (8, 5)]]
    delta = 2.0 ** 30
    rng = np.random.default_rng(21)
    for fold in (True, False):
        osh = OB.Shape(S, heads * dh, heads, dh, 64, T, lanes, 1.0, token_fold=fold)
        assert osh.folding == fold and osh.n_head == 2 and osh.KB == 8
        for lane, reqs in enumerate(lanes):
            layer = OB.BertLayer.__new__(OB.BertLayer)
            layer.ev, layer.sh, layer.lane, layer.delta, layer.ck = _EncEvaluator(), osh, lane, delta, _EncCkks()
            layer.bootstrap_all = lambda cts: [_Enc(c.value() * delta, 20, delta) for c in cts]
            toks = {name: [rng.normal(0, 0.5, (L, heads * dh)) for (_, L) in reqs] for name in "qkv"}

            def pack(x):
                # head layout: feature h*dh + k in ciphertext k // KB, block (k % KB) * H2 + h
                out = np.zeros((osh.n_head, S))
                for (o, L), xr in zip(reqs, x):
                    for h in range(heads):
                        for k in range(dh):
                            c, blk = k // osh.KB, (k % osh.KB) * osh.H2 + h
                            out[c, blk * T + o:blk * T + o + L] = xr[:, h * dh + k]
                            out[c, blk * T + o + L:blk * T + o + 2 * L] = xr[:, h * dh + k]
                return [_Enc(v * delta, 20, delta) for v in out]
            o = layer.attention(pack(toks["q"]), pack(toks["k"]), pack(toks["v"]))
            got = [c.value() for c in o]
            for r, (o_r, L) in enumerate(reqs):
                for h in range(heads):
                    sl = slice(h * dh, (h + 1) * dh)
                    s = toks["q"][r][:, sl] @ toks["k"][r][:, sl].T / np.sqrt(dh)
                    e = NB.nexus_exp(s)
                    p = e * (NB.nexus_inverse(0.01 * e.sum(axis=1, keepdims=True)) * 0.01)
                    want = p @ toks["v"][r][:, sl]
                    for k in range(dh):
                        c, blk = k // osh.KB, (k % osh.KB) * osh.H2 + h
                        assert np.allclose(got[c][blk * T + o_r:blk * T + o_r + L], want[:, k], rtol=1e-6,
                                           atol=1e-9), (fold, lane, r, h, k)


def test_layer_forward_slot_algebra(monkeypatch):
    """The oracle's whole layer (BertLayerT::forward) on exact encoded slot
    values, with the token fold on and off: the masked residual input, Q and
    K folded and unfolded (K's copies rebuilt), the attention, the folded
    residual bootstraps and LayerNorms (the halves' feature sums), the folded
    FFN and the output unfold.  Bootstraps keep the value; exp, inverse,
    invert_sqrt and GELU are NEXUS's approximations on decoded values.  The
    first token copies of the output equal the FP64 layer with the same
    approximations (nexus_gb300.bert.layer_reference)."""
    from oracle import bert as OB
    S = 512
    sh = NB.BertShape(hidden=32, heads=2, head_dim=16, ffn=64, T=32, lanes=[[(0, 10)], [(0, 3), (6, 7)]])
    w = NB.random_weights(sh, np.random.default_rng(3), std=0.2)
    delta = 2.0 ** 30
    monkeypatch.setattr(OB.L, "gelu", lambda ck, c: _Enc(NB.nexus_gelu(c.value()) * c.scale, c.limbs - 18, c.scale))
    rng = np.random.default_rng(4)
    tokens = [[rng.normal(0, 1, (L, sh.hidden)) for (_, L) in lane] for lane in sh.lanes]
    for fold in (True, False):
        osh = OB.Shape(S, sh.hidden, sh.heads, sh.head_dim, sh.ffn, sh.T, sh.lanes, 1.0, token_fold=fold)
        assert osh.folding == fold and (osh.n_hid, osh.n_head, osh.n_ffn) == (2, 2, 4)
        assert osh.copy_shifts == [7, 10]
        for lane in range(len(sh.lanes)):
            layer = OB.BertLayer.__new__(OB.BertLayer)
            layer.ev, layer.sh, layer.w, layer.lane, layer.delta = _EncEvaluator(), osh, w, lane, delta
            layer.ck = _EncCkks()
            layer.bootstrap_all = lambda cts: [_Enc(c.value() * delta, 20, delta) for c in cts]
            x = [_Enc(v * delta, 20, delta) for v in NB.pack_lane(sh, S, lane, tokens[lane])]
            out = layer.forward(x)
            got = NB.unpack_lane(sh, S, lane, np.stack([c.value() for c in out]))
            for g, r in zip(got, NB.layer_reference(sh, w, tokens[lane])):
                assert np.allclose(g, r, rtol=1e-6, atol=1e-8), (fold, lane, float(np.max(np.abs(g - r))))
