"""The encrypted BERT encoder layer restated on the oracle -- TEST
INFRASTRUCTURE (the checker of nexus_gb300/csrc/bert.cu; never shipped or
timed as the product).

The layer has no counterpart in the NEXUS tree (its drivers run one operator
at a time, src/main.cpp:25-27, and it has no ciphertext x ciphertext product);
this is the operation sequence the engine defines, written once more over the
oracle's SEAL restatement (nexus_l3.Evaluator) so that every word can be
compared.  Its pieces are NEXUS's own: CKKSEvaluator::exp and ::inverse in the
softmax sequence of src/softmax.cpp:6-42, ::invert_sqrt in the LayerNorm
sequence of src/layer_norm.cpp:6-33, GeLUEvaluator::gelu (src/gelu.cpp:5-111)
and Bootstrapper::bootstrap_3 (oracle/bootstrap.py).

Packing (the engine's): slot j*T + t of a ciphertext is feature block j at
token slot t; a lane packs requests (o_r, L_r) with tokens at o_r + i and
o_r + L_r + i.  std layout: feature f in ciphertext f // NB, block f % NB;
head layout: feature h*dh + k in ciphertext k // KB, block (k % KB)*H2 + h.
With the token fold (BertShape::token_fold), the Q, K, output, FFN1 and FFN2
maps and the residual input write the lower half of each token block only,
and two ciphertexts 2i, 2i+1 become y_2i + rot(y_2i+1, -T/2): Q and K
through their bootstrap, the hidden and FFN activations from the output
projection to the layer's output; an unfold gives 2i as the folded one and
2i+1 as its rotation by T/2 (Q at QK_LIMBS; K one level above it, with every
request's second token copy in the upper half rebuilt by masked rotations),
the attention's scores of offsets 2p and 2p + 1 go folded through their exp
and the probabilities (each half's row sum adds the other half of its own
block), and LayerNorm on folded ciphertexts adds the halves' sums with one
more rotation.
"""
from __future__ import annotations

import math

import numpy as np

from . import bootstrap as B
from . import nexus_l3 as L

LT_Q, LT_K, LT_V, LT_O, LT_1, LT_2 = range(6)
# the V projection reads its input at 4 limbs and lands at the 3 limbs the
# attention takes V at: Q and K are refreshed, V is not (kVInLimbs, bert.h)
V_IN_LIMBS = 4
# the level the attention takes Q and K at (kQKLimbs, bert.h)
QK_LIMBS = 14


def _pow2_ceil(v):
    p = 1
    while p < v:
        p <<= 1
    return p


class Shape:
    def __init__(self, slots, hidden, heads, head_dim, ffn, T, lanes, boot_shrink, boot_pack=True, rowsum_shrink=2.0,
                 token_fold=True):
        self.S, self.hidden, self.heads, self.head_dim, self.ffn, self.T = slots, hidden, heads, head_dim, ffn, T
        self.lanes = [list(l) for l in lanes]
        self.boot_shrink = float(boot_shrink)
        self.rowsum_shrink = float(rowsum_shrink)
        self.boot_pack = bool(boot_pack)
        self.NB = slots // T
        self.H2 = _pow2_ceil(heads)
        self.KB = self.NB // self.H2
        self.n_head = -(-head_dim // self.KB)
        self.n_hid = -(-hidden // self.NB)
        self.n_ffn = -(-ffn // self.NB)
        self.Lmax = max(Lr for lane in lanes for (_, Lr) in lane)
        self.G = int(math.ceil(math.sqrt(self.Lmax)))
        self.Glt = int(math.ceil(math.sqrt(self.NB)))
        # BertShape::derive: the fold needs every request's tokens in [0, T/2)
        self.token_fold = bool(token_fold)
        self.fold_ok = all(o + Lr <= T // 2 for lane in lanes for (o, Lr) in lane)
        # lengths of the requests whose second token copy reaches the upper half
        self.copy_shifts = sorted({Lr for lane in lanes for (o, Lr) in lane if o + 2 * Lr > T // 2})

    @property
    def folding(self):
        return self.token_fold and self.fold_ok

    def rotation_steps(self):
        v = []

        def push(s):
            s %= self.S
            if s and s not in v:
                v.append(s)
        for b in range(1, self.Glt):
            push(b * self.T)
        g = 1
        while g * self.Glt < self.NB:
            push(g * self.Glt * self.T)
            g += 1
        for b in range(1, self.G):
            push(b)
        g = 1
        while g * self.G < self.Lmax:
            push(g * self.G)
            push(-g * self.G)
            g += 1
        m = 1
        while m < self.KB:
            push(self.H2 * self.T * m)
            m <<= 1
        m = 1
        while m < self.NB:
            push(self.T * m)
            m <<= 1
        if self.fold_ok:
            push(self.T // 2)
            push(-self.T // 2)
            for s in self.copy_shifts:
                push(-s)
        return v


class BertLayer:
    """The engine's BertLayerT for one lane, on the oracle."""

    def __init__(self, ev: L.Evaluator, bs, shape: Shape, w: dict, lane: int):
        self.ev, self.bs, self.sh, self.w, self.lane = ev, bs, shape, w, lane
        self.delta = float(bs.final_scale)
        self.ck = L.CKKSEvaluator(ev, self.delta)

    # -- linear maps -----------------------------------------------------------
    def _in_count(self, which):
        sh = self.sh
        return sh.n_head if which == LT_O else (sh.n_ffn if which == LT_2 else sh.n_hid)

    def _out_count(self, which):
        sh = self.sh
        return sh.n_head if which <= LT_V else (sh.n_ffn if which == LT_1 else sh.n_hid)

    def _head_feature(self, ct, block):
        sh = self.sh
        h, k = block % sh.H2, ct * sh.KB + block // sh.H2
        return -1 if h >= sh.heads or k >= sh.head_dim else h * sh.head_dim + k

    def _in_feature(self, which, ct, block):
        if which == LT_O:
            return self._head_feature(ct, block)
        f = ct * self.sh.NB + block
        return f if f < (self.sh.ffn if which == LT_2 else self.sh.hidden) else -1

    def _out_feature(self, which, ct, block):
        if which <= LT_V:
            return self._head_feature(ct, block)
        f = ct * self.sh.NB + block
        return f if f < (self.sh.ffn if which == LT_1 else self.sh.hidden) else -1

    def _weights(self, which):
        return self.w[("wq", "wk", "wv", "wo", "w1", "w2")[which]]

    def _bias(self, which):
        return self.w[("bq", "bk", "bv", "bo", "b1", "b2")[which]]

    def _diag(self, which, a, b, d, lower_half=False):
        """diagonal d of block (a -> b), divided by boot_shrink, or None when
        zero; lower_half: on token slots [0, T/2) of each block only"""
        sh = self.sh
        W = self._weights(which)
        vals = np.zeros(sh.NB)
        nz = False
        for j in range(sh.NB):
            fo, fi = self._out_feature(which, b, j), self._in_feature(which, a, (j + d) % sh.NB)
            if fo >= 0 and fi >= 0:
                vals[j] = W[fi, fo] / sh.boot_shrink
                nz = True
        if not nz:
            return None
        g = d // sh.Glt
        vals = np.roll(vals, g * sh.Glt)       # pre-rotated by the giant step
        return self._spread(vals, lower_half)

    def _spread(self, per_block, lower_half):
        """one value per block on every token slot of it (the lower half only)"""
        sh = self.sh
        v = np.repeat(per_block, sh.T).reshape(sh.NB, sh.T)
        if lower_half:
            v[:, sh.T // 2:] = 0.0
        return v.ravel()

    def project(self, x, which, lower_half=False):
        ev, sh = self.ev, self.sh
        l = x[0].limbs
        in_scale = x[0].scale
        dscale = float(ev.q[l - 1]) * self.delta / in_scale
        baby = [[xa] + [ev.rotate(xa, b * sh.T) for b in range(1, sh.Glt)] for xa in x]
        y = []
        for b in range(self._out_count(which)):
            acc = None
            g = 0
            while g * sh.Glt < sh.NB:
                giant = None
                for a in range(len(x)):
                    for bb in range(sh.Glt):
                        d = g * sh.Glt + bb
                        if d >= sh.NB:
                            break
                        v = self._diag(which, a, b, d, lower_half)
                        if v is None:
                            continue
                        t = ev.multiply_plain(baby[a][bb], ev.encode(v, dscale, l))
                        giant = t if giant is None else ev.add(giant, t)
                if giant is not None:
                    t = ev.rotate(giant, g * sh.Glt * sh.T) if g else giant
                    acc = t if acc is None else ev.add(acc, t)
                g += 1
            acc = ev.rescale(acc)
            acc.scale = self.delta / sh.boot_shrink
            per_block = np.zeros(sh.NB)
            bv = self._bias(which)
            for j in range(sh.NB):
                f = self._out_feature(which, b, j)
                if f >= 0:
                    per_block[j] = bv[f]
            acc = ev.add_plain(acc, ev.encode(self._spread(per_block, lower_half), acc.scale, acc.limbs))
            y.append(acc)
        return y

    def fold_halves(self, x):
        """BertLayerT::fold_halves: x[2i] + rot(x[2i+1], -T/2), an odd last one alone."""
        ev, sh = self.ev, self.sh
        out = []
        for i in range(0, len(x), 2):
            out.append(ev.add(x[i], ev.rotate(x[i + 1], sh.S - sh.T // 2)) if i + 1 < len(x) else x[i])
        return out

    def unfold_halves(self, x, count):
        """BertLayerT::unfold_halves: ciphertext 2i is x[i], 2i+1 is rot(x[i], T/2)."""
        assert len(x) == (count + 1) // 2
        return [x[i // 2] if i % 2 == 0 else self.ev.rotate(x[i // 2], self.sh.T // 2) for i in range(count)]

    def _copy_mask(self, shift, limbs):
        """BertLayerT::copy_masks for this lane: the lower half of every block
        (shift 0), or the tokens of the requests of length `shift` whose copy
        lies in the upper half; at the scale of the prime the rescale drops."""
        sh = self.sh
        half = sh.T // 2
        block = np.zeros(sh.T)
        if shift == 0:
            block[:half] = 1.0
        else:
            for (o, Lr) in sh.lanes[self.lane]:
                if Lr == shift:
                    block[max(o, half - shift):o + Lr] = 1.0
        return self.ev.encode(np.tile(block, sh.NB), float(self.ev.q[limbs - 1]), limbs)

    def unfold_copies(self, x, count):
        """BertLayerT::unfold_copies: unfold_halves with every request's
        second token copy in the upper half rebuilt from its tokens."""
        ev, sh = self.ev, self.sh
        assert len(x) == (count + 1) // 2
        limbs = x[0].limbs
        out = []
        for i in range(count):
            h = ev.rotate(x[i // 2], sh.T // 2) if i % 2 else x[i // 2]
            acc = ev.rescale(ev.multiply_plain(h, self._copy_mask(0, limbs)))
            for s in sh.copy_shifts:
                t = ev.rescale(ev.multiply_plain(h, self._copy_mask(s, limbs)))
                acc = ev.add(acc, ev.rotate(t, sh.S - s))
            out.append(acc)
        return out

    # -- helpers ------------------------------------------------------------------
    def exact_scale_const(self, ct, value, target, lower_half=False):
        ev = self.ev
        q = float(ev.q[ct.limbs - 1])
        sc = q * target / ct.scale
        if lower_half:
            p = ev.encode(self._spread(np.full(self.sh.NB, value), True), sc, ct.limbs)
        else:
            p = ev.encode_scalar(value, sc, ct.limbs)
        ct = ev.rescale(ev.multiply_plain(ct, p))
        ct.scale = target
        return ct

    def shrink_for_bootstrap(self, cts, lower_half=False):
        out = []
        for c in cts:
            c = self.exact_scale_const(c, 1.0 / self.sh.boot_shrink, self.delta, lower_half)
            c.scale = self.delta / self.sh.boot_shrink
            out.append(c)
        return out

    def bootstrap_all(self, cts):
        """BertLayerT::bootstrap_all: every ciphertext refreshed at one limb;
        with boot_pack, ciphertexts 2i and 2i + 1 share one bootstrap
        (bootstrap.bootstrap_real_pair); a trailing odd one is a pair whose
        second member is zero (its scale doubled, then z + conj(z))."""
        ev = self.ev
        cts = [ev.mod_switch_to(c, 1) for c in cts]
        if not self.sh.boot_pack:
            return [self.bs.bootstrap_3(c) for c in cts]
        out = []
        for i in range(0, len(cts) - 1, 2):
            out.extend(B.bootstrap_real_pair(self.bs, cts[i], cts[i + 1]))
        if len(cts) % 2:
            z = L.Ct(cts[-1].data, cts[-1].scale * 2.0)
            r = self.bs.bootstrap_3(z)
            out.append(ev.add(r, ev.conjugate(r)))
        return out

    def _mask(self, delta, kind, limbs, scale):
        sh = self.sh
        reqs = sh.lanes[self.lane]
        v = np.zeros(sh.S)
        inv_sqrt = 1.0 / math.sqrt(sh.head_dim)
        for j in range(sh.NB):
            head_ok = (j % sh.H2) < sh.heads
            for t in range(sh.T):
                ok = head_ok and any(delta < Lr and o <= t < o + Lr for (o, Lr) in reqs)
                v[j * sh.T + t] = (inv_sqrt if ok else 0.0) if kind == 0 else (0.0 if ok else -128.0)
        sc = float(self.ev.q[limbs - 1]) if kind == 0 else scale
        return self.ev.encode(v, sc, limbs)

    def _fold_mask(self, pair, limbs, scale):
        """BertLayerT::fold_masks for this lane: the -128 masks of offsets
        2 pair (lower half) and 2 pair + 1 (upper half) in one plaintext."""
        sh = self.sh
        reqs = sh.lanes[self.lane]
        half = sh.T // 2
        v = np.zeros(sh.S)
        for j in range(sh.NB):
            head_ok = (j % sh.H2) < sh.heads
            for t in range(sh.T):
                d, tt = (2 * pair, t) if t < half else (2 * pair + 1, t - half)
                ok = head_ok and d < sh.Lmax and any(d < Lr and o <= tt < o + Lr for (o, Lr) in reqs)
                v[j * sh.T + t] = 0.0 if ok else -128.0
        return self.ev.encode(v, scale, limbs)

    def _half(self, value, upper, limbs, scale):
        """BertLayerT::half_plain: value on one half of every token block."""
        sh = self.sh
        block = np.zeros(sh.T)
        block[sh.T // 2:] = value if upper else 0.0
        block[:sh.T // 2] = 0.0 if upper else value
        return self.ev.encode(np.tile(block, sh.NB), scale, limbs)

    # -- blocks -----------------------------------------------------------------
    def attention(self, q, k, v):
        ev, sh, ck = self.ev, self.sh, self.ck
        nh, G, Lm, S = sh.n_head, sh.G, sh.Lmax, sh.S
        e_limbs = 4
        q = [ev.mod_switch_to(c, QK_LIMBS) for c in q]
        k = [ev.mod_switch_to(c, QK_LIMBS) for c in k]
        v = [ev.mod_switch_to(c, e_limbs - 1) for c in v]
        n_g = -(-Lm // G)
        kb = [[c] + [ev.rotate(c, b) for b in range(1, G)] for c in k]
        vb = [[c] + [ev.rotate(c, b) for b in range(1, G)] for c in v]
        qg = [[c] + [ev.rotate(c, S - g * G) for g in range(1, n_g)] for c in q]
        e = []
        for d in range(Lm):
            g, b = divmod(d, G)
            acc = None
            for c in range(nh):
                t = ev.multiply(qg[c][g], kb[c][b])
                acc = t if acc is None else ev.add(acc, t)
            acc = ev.rescale(ev.relinearize(acc))
            if g:
                acc = ev.rotate(acc, g * G)
            acc = ev.rescale(ev.multiply_plain(acc, self._mask(d, 0, acc.limbs, acc.scale)))
            e.append(acc)
        if sh.folding:
            # offsets 2p and 2p + 1 in the two halves of one ciphertext
            e = self.fold_halves(e)
        # the sum over the KB blocks of each head, once per ciphertext after
        # the zeroing mask and the fold (it commutes with both), then -128
        summed = []
        for p, c in enumerate(e):
            m = 1
            while m < sh.KB:
                c = ev.add(c, ev.rotate(c, sh.H2 * sh.T * m))
                m <<= 1
            mask = self._fold_mask(p, c.limbs, c.scale) if sh.folding else self._mask(p, 1, c.limbs, c.scale)
            summed.append(ev.add_plain(c, mask))
        e = [ck.exp(c) for c in summed]
        total = e[0]
        for c in e[1:]:
            total = ev.add(total, c)
        cst = 0.01 / sh.rowsum_shrink
        delta = ev.encode_scalar(cst, total.scale, total.limbs)
        if sh.folding:
            # each half adds the other half of its own block
            up = ev.multiply_plain(ev.rotate(total, sh.T // 2), self._half(cst, False, total.limbs, total.scale))
            down = ev.multiply_plain(ev.rotate(total, S - sh.T // 2),
                                     self._half(cst, True, total.limbs, total.scale))
            total = ev.add(ev.add(ev.multiply_plain(total, delta), up), down)
        else:
            total = ev.multiply_plain(total, delta)
        total = ev.rescale(total)
        total.scale /= sh.rowsum_shrink
        inv = ck.inverse(self.bootstrap_all([total])[0])
        inv = ev.rescale(ev.multiply_plain(inv, ev.encode_scalar(0.01, inv.scale, inv.limbs)))
        inv = ev.mod_switch_to(inv, e[0].limbs)
        p = [ev.rescale(ev.relinearize(ev.multiply(ed, inv))) for ed in e]
        if sh.folding:
            p = self.unfold_halves(p, Lm)
        pg = [[(ev.rotate(p[g * G + b], S - g * G) if g else p[b]) for b in range(G) if g * G + b < Lm]
              for g in range(n_g)]
        o = []
        for c in range(nh):
            acc = None
            for g in range(n_g):
                part = None
                for b in range(len(pg[g])):
                    t = ev.multiply(pg[g][b], vb[c][b])
                    part = t if part is None else ev.add(part, t)
                part = ev.rescale(ev.relinearize(part))
                if g:
                    part = ev.rotate(part, g * G)
                acc = part if acc is None else ev.add(acc, part)
            o.append(acc)
        return o

    def layer_norm(self, x, folded=False):
        ev, sh = self.ev, self.sh
        total = None
        for c in x:
            t = ev.rescale(ev.relinearize(ev.square(c)))
            total = t if total is None else ev.add(total, t)
        m = 1
        while m < sh.NB:
            total = ev.add(total, ev.rotate(total, sh.T * m))
            m <<= 1
        if folded:
            total = ev.add(total, ev.rotate(total, sh.T // 2))
        total = ev.rescale(ev.multiply_plain(total, ev.encode_scalar(1.0 / sh.hidden, total.scale, total.limbs)))
        r = self.ck.invert_sqrt(total, 4, 2)
        return [ev.rescale(ev.relinearize(ev.multiply(ev.mod_switch_to(c, r.limbs), r))) for c in x]

    def forward(self, x, trace=None):
        """x: n_hid ciphertexts of this lane; returns the layer's output.
        trace, a dict, receives every stage's ciphertexts."""
        ev, sh = self.ev, self.sh
        rec = (lambda k, v: trace.__setitem__(k, v)) if trace is not None else (lambda k, v: None)
        fold = sh.folding
        x_res = [ev.mod_switch_to(c, 1) for c in self.shrink_for_bootstrap(x, fold)]
        x2 = [ev.mod_switch_to(c, 2) for c in x]
        x4 = [ev.mod_switch_to(c, V_IN_LIMBS) for c in x]
        q, k, v = self.project(x2, LT_Q, fold), self.project(x2, LT_K, fold), self.project(x4, LT_V)
        rec("qkv", q + k + v)
        if fold:
            q, k = self.fold_halves(q), self.fold_halves(k)
        nq = len(q)
        qk = self.bootstrap_all(q + k)
        rec("qk_boot", qk)
        q, k = qk[:nq], qk[nq:]
        if fold:
            q = self.unfold_halves([ev.mod_switch_to(c, QK_LIMBS) for c in q], sh.n_head)
            k = self.unfold_copies([ev.mod_switch_to(c, QK_LIMBS + 1) for c in k], sh.n_head)
        rec("qkv_boot", q + k + v)
        o = self.attention(q, k, v)
        rec("attention", o)
        a = self.project(o, LT_O, fold)
        for c in range(sh.n_hid):
            a[c].scale = x_res[c].scale
            a[c] = ev.add(a[c], x_res[c])
        if fold:
            a = self.fold_halves(a)
        a = self.bootstrap_all(a)
        rec("residual1_boot", a)
        a = self.layer_norm(a, fold)
        rec("ln1", a)
        y_res = [ev.mod_switch_to(c, 1) for c in self.shrink_for_bootstrap(a)]
        a2 = [ev.mod_switch_to(c, 2) for c in a]
        if fold:
            a2 = self.unfold_halves(a2, sh.n_hid)
        h = self.project(a2, LT_1, fold)
        if fold:
            h = self.fold_halves(h)
        h = self.bootstrap_all(h)
        rec("ffn1_boot", h)
        h = [L.gelu(self.ck, c) for c in h]
        rec("gelu", h)
        if fold:
            h = self.unfold_halves(h, sh.n_ffn)
        f = self.project(h, LT_2, fold)
        if fold:
            f = self.fold_halves(f)
        for c in range(len(f)):
            f[c].scale = y_res[c].scale
            f[c] = ev.add(f[c], y_res[c])
        f = self.bootstrap_all(f)
        rec("residual2_boot", f)
        out = self.layer_norm(f, fold)
        if fold:
            out = self.unfold_halves(out, sh.n_hid)
        rec("output", out)
        return out
