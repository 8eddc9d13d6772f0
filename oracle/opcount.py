"""Operation counts of the oracle's bootstrap -- TEST / MEASUREMENT INFRASTRUCTURE.

The control flow of Bootstrapper.cpp depends only on levels and scales, never
on ciphertext words, so running the oracle restatement (bootstrap.py) over an
evaluator that tracks only (size, limbs, scale) yields the exact sequence of
ring operations a full-size bootstrap performs.  Each operation is recorded
as (name, limbs); the CPU baseline multiplies these counts by the oracle's
measured time per operation at the same ring size.
"""
from __future__ import annotations

from collections import Counter

import numpy as np

from . import bootstrap as B
from . import nexus_l3 as L
from . import pyoracle as po


def _ct(size, limbs, scale):
    return L.Ct(np.zeros((size, limbs, 0), dtype=np.uint64), scale)


class CountingEvaluator(L.Evaluator):
    """nexus_l3.Evaluator semantics (levels, scales, errors) without data."""

    def __init__(self, moduli, log_n: int, galois_elts):
        self.oc = None
        self.n = 1 << log_n
        self.log_n = log_n
        self.slots = self.n // 2
        self.top = len(moduli) - 1
        self.q = [int(q) for q in moduli]
        self.relin_key = True
        self.galois_keys = {int(e): True for e in galois_elts}
        self._bits = {}
        self.ops = Counter()

    def _rec(self, name, limbs):
        self.ops[(name, int(limbs))] += 1

    # encoding
    def encode(self, values, scale, limbs=None):
        limbs = limbs or self.top
        self._check_scale(scale, limbs)
        self._rec("encode", limbs)
        return L.Pt(scale, data=np.zeros((limbs, 0), dtype=np.uint64))

    def encode_scalar(self, value, scale, limbs=None):
        limbs = limbs or self.top
        return L.Pt(scale, per_limb=np.zeros(limbs, dtype=np.uint64))

    def encode_then_drop(self, values, scale, limbs):
        if np.ndim(values) == 0:
            return L.Pt(scale, per_limb=np.zeros(limbs, dtype=np.uint64))
        self._rec("encode", limbs)
        return L.Pt(scale, data=np.zeros((limbs, 0), dtype=np.uint64))

    # arithmetic
    def rescale(self, ct):
        if ct.limbs < 2:
            raise ValueError("end of modulus switching chain reached")
        scale = ct.scale / float(self.q[ct.limbs - 1])
        self._check_scale(scale, ct.limbs - 1)
        self._rec("rescale", ct.limbs)
        return _ct(ct.data.shape[0], ct.limbs - 1, scale)

    def multiply(self, a, b):
        self._same_level(a, b)
        scale = a.scale * b.scale
        self._check_scale(scale, a.limbs)
        self._rec("tensor", a.limbs)
        return _ct(3, a.limbs, scale)

    def relinearize(self, ct):
        if ct.data.shape[0] == 2:
            return ct.copy()
        self._rec("relin", ct.limbs)
        return _ct(2, ct.limbs, ct.scale)

    def add(self, a, b):
        self._same_level(a, b)
        if not L.are_close(a.scale, b.scale):
            raise ValueError("scale mismatch")
        self._rec("add", a.limbs)
        return _ct(max(a.data.shape[0], b.data.shape[0]), a.limbs, a.scale)

    def sub(self, a, b):
        return self.add(a, b)

    def negate(self, a):
        self._rec("add", a.limbs)
        return a.copy()

    def _plain_arith(self, ct, pt, sub):
        if ct.limbs != pt.limbs:
            raise ValueError("encrypted and plain parameter mismatch")
        if not L.are_close(ct.scale, pt.scale):
            raise ValueError("scale mismatch")
        self._rec("add", 1)
        return ct.copy()

    def multiply_plain(self, ct, pt):
        if ct.limbs != pt.limbs:
            raise ValueError("encrypted and plain parameter mismatch")
        scale = ct.scale * pt.scale
        self._check_scale(scale, ct.limbs)
        self._rec("mul_plain", ct.limbs)
        return _ct(ct.data.shape[0], ct.limbs, scale)

    def apply_galois(self, ct, elt):
        if elt not in self.galois_keys:
            raise ValueError("Galois key not present")
        self._rec("galois", ct.limbs)
        return ct.copy()

    def rotate(self, ct, steps):
        if steps == 0:
            return ct.copy()
        elt = po.galois_elt_from_step(self.log_n, steps)
        if elt in self.galois_keys:
            return self.apply_galois(ct, elt)
        out = ct
        for st in L.naf(steps):
            if abs(st) != (self.n >> 1):
                out = self.rotate(out, st)
        return out

    def conjugate(self, ct):
        return self.apply_galois(ct, 2 * self.n - 1)


class _CountingBootstrapper(B.Bootstrapper):
    def modraise_inplace(self, ct):
        if ct.limbs != 1:
            raise ValueError("Ciphertexts in the lowest level are supported only!")
        self.ev._rec("modraise", self.ev.top)
        return _ct(2, self.ev.top, ct.scale)


def bootstrap_op_counts(moduli, log_n: int, logn: int, table: dict, loge=10, boundary_k=25, deg=59,
                        scale_factor=2, inverse_deg=1, scale=2.0 ** 46) -> Counter:
    """(name, limbs) -> count for one bootstrap_3 of a one-limb ciphertext at `scale`."""
    log_nh = log_n - 1
    steps = B.rot_key_steps_3(logn, log_nh)
    ev = CountingEvaluator(moduli, log_n, [po.galois_elt_from_step(log_n, s) for s in steps])
    bs = _CountingBootstrapper(ev, loge, logn, log_nh, len(moduli) - 2, scale, boundary_k, deg, scale_factor,
                               inverse_deg, table)
    # diagonal values do not change the operation sequence: zeros of the right shapes
    z = (np.zeros(1 << logn), np.zeros(1 << logn))
    f = [(1 << d) - 1 for d in B.split3_fwd(logn)]
    i = [(1 << d) - 1 for d in B.split3_inv(logn)]
    bs.fftcoeff = ([z] * (2 * f[0] + 1), [z] * (2 * f[1] + 1), [z] * (f[2] + 1))
    bs.invfftcoeff = ([z] * (i[0] + 1), [z] * (2 * i[1] + 1), [z] * (2 * i[2] + 1))
    bs._mul_vec = lambda ct, re, im: ev.multiply_plain(ct, ev.encode_then_drop(np.zeros(1), ct.scale, ct.limbs))
    out = bs.bootstrap_3(_ct(2, 1, scale))
    ev.ops[("output_limbs", out.limbs)] += 1
    return ev.ops
