"""Encrypted BERT encoder layer: shapes, client-side packing and the FP64
references the decrypted outputs are compared with.

The layer itself runs in the engine (csrc/bert.cu, nexus_bert_layer_*); see
its header comment for the packing.  In short: slot ``j*T + t`` of a
ciphertext holds feature block ``j`` at token slot ``t``; a lane packs several
requests into the T token slots, request r at ``[o_r, o_r + 2 L_r)`` with its
tokens at ``o_r + i`` and again at ``o_r + L_r + i``.

The FP64 reference evaluates the same approximations NEXUS's operators use
(``(1 + x/128)^128`` for exp, the product form of the inverse, the line +
Newton + Goldschmidt inverse square root, the sign-polynomial GELU), so the
gap to it measures the encrypted evaluation's error; the exact reference
(softmax, 1/sqrt, tanh GELU) is reported beside it.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from ._lib import check, lib


@dataclass
class BertShape:
    hidden: int = 768
    heads: int = 12
    head_dim: int = 64
    ffn: int = 3072
    T: int = 256
    # per lane, requests as (first token slot, tokens)
    lanes: list = field(default_factory=lambda: [[(0, 128)], [(0, 32), (64, 64)]])
    boot_shrink: float = 1.0
    # two ciphertexts per bootstrap (c0 + i c1, separated by a conjugation)
    boot_pack: bool = True
    # two ciphertexts in one (the halves of each token block) for Q and K
    # through their bootstrap and for the activations after the attention,
    # when every request's tokens lie in [0, T/2)
    token_fold: bool = True

    def blocks(self, slots: int) -> int:
        return slots // self.T

    def n_hid(self, slots: int) -> int:
        return -(-self.hidden // self.blocks(slots))

    def requests(self):
        """(lane, first slot, tokens) of every request, in lane order."""
        return [(li, o, L) for li, lane in enumerate(self.lanes) for (o, L) in lane]


BERT_BASE = BertShape()


def random_weights(shape: BertShape, rng: np.random.Generator, std: float = 0.02) -> dict:
    d, f = shape.hidden, shape.ffn
    w = {k: rng.normal(0, std, (d, d)) for k in ("wq", "wk", "wv", "wo")}
    w["w1"] = rng.normal(0, std, (d, f))
    w["w2"] = rng.normal(0, std, (f, d))
    for k, n in (("bq", d), ("bk", d), ("bv", d), ("bo", d), ("b1", f), ("b2", d)):
        w[k] = rng.normal(0, std, n)
    return w


def flat_weights(w: dict) -> np.ndarray:
    return np.concatenate([np.ravel(w[k]) for k in ("wq", "wk", "wv", "wo", "w1", "w2",
                                                     "bq", "bk", "bv", "bo", "b1", "b2")]).astype(np.float64)


def pack_lane(shape: BertShape, slots: int, lane: int, tokens: list) -> np.ndarray:
    """Slot vectors [n_hid][slots] of one lane: tokens[r] is request r's
    [L_r][hidden] input, placed at both token copies."""
    nb = shape.blocks(slots)
    out = np.zeros((shape.n_hid(slots), slots))
    for (o, L), x in zip(shape.lanes[lane], tokens):
        x = np.asarray(x)
        assert x.shape == (L, shape.hidden)
        for f in range(shape.hidden):
            c, j = divmod(f, nb)
            base = j * shape.T + o
            out[c, base:base + L] = x[:, f]
            out[c, base + L:base + 2 * L] = x[:, f]
    return out


def unpack_lane(shape: BertShape, slots: int, lane: int, vecs: np.ndarray) -> list:
    """Inverse of pack_lane for the first token copies: [L_r][hidden] per request."""
    nb = shape.blocks(slots)
    res = []
    for (o, L) in shape.lanes[lane]:
        y = np.zeros((L, shape.hidden))
        for f in range(shape.hidden):
            c, j = divmod(f, nb)
            y[:, f] = vecs[c, j * shape.T + o:j * shape.T + o + L]
        res.append(y)
    return res


# ----------------------------------------------------------------------------- FP64 references

def nexus_exp(x):
    """CKKSEvaluator::exp (src/ckks_evaluator.cpp:534-548): (1 + x/128)^128."""
    y = x * 0.0078125 + 1.0
    for _ in range(7):
        y = y * y
    return y


def nexus_inverse(x, iters: int = 4):
    """CKKSEvaluator::inverse (src/ckks_evaluator.cpp:487-509): prod (1 + y^(2^i)), y = 1 - x."""
    y = 1.0 - x
    res = 1.0 + y
    for _ in range(iters):
        y = y * y
        res = res * (1.0 + y)
    return res


def nexus_invert_sqrt(x, d_newt: int = 4, d_gold: int = 2):
    """CKKSEvaluator::invert_sqrt (src/ckks_evaluator.cpp:366-485): the line
    initGuess, d_newt Newton steps r <- r (3 - x r^2) / 2, then d_gold
    Goldschmidt steps on (sqrt, 1/(2 sqrt))."""
    r = -1.29054537e-04 * x + 1.29054537e-01
    for _ in range(d_newt):
        r = r * (3.0 - x * r * r) * 0.5
    s = x * r
    h = r * 0.5
    for _ in range(d_gold):
        rr = 0.5 - s * h
        s = s + s * rr
        h = h + h * rr
    return h * 2.0


def _odd_poly(coeffs, scale, x):
    return sum(c / scale * x ** i for i, c in enumerate(coeffs) if c)


def nexus_sgn(x, d_g: int = 2, d_f: int = 2, sgn_factor: float = 0.5):
    """CKKSEvaluator::sgn_eval (src/ckks_evaluator.cpp:181-212): d_g rounds of
    the g4 polynomial then d_f of f4, the last round of each scaled by sgn_factor."""
    f4 = [0, 315, 0, -420, 0, 378, 0, -180, 0, 35]
    g4 = [0, 5850, 0, -34974, 0, 97015, 0, -113492, 0, 46623]
    for i in range(d_g):
        x = _odd_poly(g4, 1 << 10, x) * (sgn_factor if i == d_g - 1 else 1.0)
    for i in range(d_f):
        x = _odd_poly(f4, 1 << 7, x) * (sgn_factor if i == d_f - 1 else 1.0)
    return x


def nexus_gelu(x):
    """GeLUEvaluator::gelu (src/gelu.cpp:5-111) on plain values:
    A(x) (b0 - b1) + x (b1 + 1/2), b0 = sgn((x + 3.5) / 8.5), b1 = sgn((x - 3.5) / 8.5),
    A an even polynomial in x, x^2, x^4, ..., x^12 (src/gelu.cpp:64)."""
    a = [2.25775755e-04, 0.5, 3.96880960e-01, -6.37042698e-02, 8.38841647e-03, -7.17830961e-04,
         3.49617829e-05, -7.26059653e-07]
    b0 = nexus_sgn((x + 3.5) / 8.5)
    b1 = nexus_sgn((x - 3.5) / 8.5)
    x2 = x * x
    poly = a[0] + a[1] * x + a[2] * x2 + a[3] * x2 ** 2 + a[4] * x2 ** 3 + a[5] * x2 ** 4 + a[6] * x2 ** 5 \
        + a[7] * x2 ** 6
    return poly * (b0 - b1) + x * (b1 + 0.5)


def layer_reference(shape: BertShape, w: dict, tokens: list, exact: bool = False) -> list:
    """The layer on plain values for each request's [L][hidden] input, with
    NEXUS's approximations (exact=False) or the exact functions."""
    H, dh = shape.heads, shape.head_dim
    outs = []
    for x in tokens:
        L = x.shape[0]
        q, k, v = x @ w["wq"] + w["bq"], x @ w["wk"] + w["bk"], x @ w["wv"] + w["bv"]
        o = np.zeros_like(q)
        for h in range(H):
            sl = slice(h * dh, (h + 1) * dh)
            s = q[:, sl] @ k[:, sl].T / math.sqrt(dh)
            if exact:
                e = np.exp(s - s.max(axis=1, keepdims=True))
                p = e / e.sum(axis=1, keepdims=True)
            else:
                e = nexus_exp(s)
                p = e * (nexus_inverse(0.01 * e.sum(axis=1, keepdims=True)) * 0.01)
            o[:, sl] = p @ v[:, sl]
        a = o @ w["wo"] + w["bo"] + x

        def ln(z):
            m = (z * z).sum(axis=1, keepdims=True) / shape.hidden
            return z * ((1.0 / np.sqrt(m)) if exact else nexus_invert_sqrt(m, 4, 2))
        y = ln(a)
        hdn = y @ w["w1"] + w["b1"]
        if exact:
            g = 0.5 * hdn * (1.0 + np.tanh(math.sqrt(2.0 / math.pi) * (hdn + 0.044715 * hdn ** 3)))
        else:
            g = nexus_gelu(hdn)
        outs.append(ln(y + g @ w["w2"] + w["b2"]))
    return outs


# ----------------------------------------------------------------------------- engine wrapper

class BertLayer:
    """nexus_bert_layer_* over a Bootstrapper (operators.Bootstrapper) whose
    evaluator holds the relinearization key, the bootstrapping keys and the
    Galois keys of rotation_steps()."""

    def __init__(self, bootstrapper, shape: BertShape, weights: dict):
        self.bs = bootstrapper
        self.ctx = bootstrapper.ctx
        self.shape = shape
        lanes = shape.lanes
        counts = (C.c_int * len(lanes))(*[len(lane) for lane in lanes])
        reqs = [v for lane in lanes for (o, L) in lane for v in (o, L)]
        req = (C.c_int * len(reqs))(*reqs)
        flat = flat_weights(weights)
        h = C.c_void_p()
        check(lib().nexus_bert_layer_create(bootstrapper._h, shape.hidden, shape.heads, shape.head_dim, shape.ffn,
                                            shape.T, len(lanes), counts, req, C.c_double(shape.boot_shrink),
                                            flat.ctypes.data_as(C.POINTER(C.c_double)), C.byref(h)),
              "nexus_bert_layer_create")
        self._h = h
        info = [C.c_int() for _ in range(4)]
        cached = C.c_uint64()
        check(lib().nexus_bert_layer_info(self._h, *[C.byref(i) for i in info], C.byref(cached)),
              "nexus_bert_layer_info")
        self.n_lanes, self.n_hid, self.n_head, self.n_ffn = [i.value for i in info]
        self.set_boot_pack(shape.boot_pack)
        self.set_token_fold(shape.token_fold)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nexus_bert_layer_destroy(self._h)
            self._h = None

    def rotation_steps(self) -> list:
        n = C.c_int()
        check(lib().nexus_bert_layer_rotation_steps(self._h, None, C.byref(n), 0), "nexus_bert_layer_rotation_steps")
        arr = (C.c_int * max(1, n.value))()
        check(lib().nexus_bert_layer_rotation_steps(self._h, arr, C.byref(n), n.value),
              "nexus_bert_layer_rotation_steps")
        return list(arr[:n.value])

    def cached_plaintexts(self) -> int:
        cached = C.c_uint64()
        check(lib().nexus_bert_layer_info(self._h, None, None, None, None, C.byref(cached)), "nexus_bert_layer_info")
        return cached.value

    def set_timing(self, enable: bool) -> None:
        check(lib().nexus_bert_layer_set_timing(self._h, 1 if enable else 0), "nexus_bert_layer_set_timing")

    def set_boot_pack(self, enable: bool) -> None:
        """Two ciphertexts per bootstrap (nexus_bert_layer_set_boot_pack)."""
        check(lib().nexus_bert_layer_set_boot_pack(self._h, 1 if enable else 0), "nexus_bert_layer_set_boot_pack")

    def set_token_fold(self, enable: bool) -> None:
        """Q, K and the activations after the attention folded two
        ciphertexts in one (nexus_bert_layer_set_token_fold)."""
        check(lib().nexus_bert_layer_set_token_fold(self._h, 1 if enable else 0), "nexus_bert_layer_set_token_fold")

    def stage_times(self, lockstep: bool = True, lane: int = 0) -> dict:
        """Device ms of each block of the last forward with timing on."""
        n = C.c_int()
        check(lib().nexus_bert_layer_stage_times(self._h, int(lockstep), lane, None, None, 0, C.byref(n), 0),
              "nexus_bert_layer_stage_times")
        ms = (C.c_double * max(1, n.value))()
        names = C.create_string_buffer(4096)
        check(lib().nexus_bert_layer_stage_times(self._h, int(lockstep), lane, ms, names, 4096, C.byref(n), n.value),
              "nexus_bert_layer_stage_times")
        return dict(zip(names.value.decode().split("\n"), ms[:n.value]))

    def _handles(self, cts):
        return (C.c_void_p * len(cts))(*[c.handle.value for c in cts])

    def forward(self, x: list, lockstep: bool = True) -> list:
        """x: lane-major ciphertexts [n_lanes * n_hid]; returns the same shape."""
        from .operators import Ciphertext
        assert len(x) == self.n_lanes * self.n_hid
        out = [Ciphertext(self.ctx) for _ in x]
        check(lib().nexus_bert_layer_forward(self._h, 1 if lockstep else 0, self._handles(x), self._handles(out)),
              "nexus_bert_layer_forward")
        return out

    def stage(self, stage: int, which: int, x: list, n_out_per_lane: int, lockstep: bool = True) -> list:
        from .operators import Ciphertext
        out = [Ciphertext(self.ctx) for _ in range(self.n_lanes * n_out_per_lane)]
        check(lib().nexus_bert_layer_stage(self._h, 1 if lockstep else 0, stage, which, self._handles(x),
                                           len(x) // self.n_lanes, self._handles(out), n_out_per_lane),
              "nexus_bert_layer_stage")
        return out


BERT_PROJECT, BERT_ATTENTION, BERT_LAYER_NORM, BERT_BOOTSTRAP, BERT_FOLD, BERT_UNFOLD = 0, 1, 2, 3, 4, 5
# OR-ed into a BERT_PROJECT map: written on the lower half of each token block only
BERT_LOWER_HALF = 16
