"""CPU restatement of NEXUS's operators on the oracle -- TEST INFRASTRUCTURE.

The classes below restate, call by call, the SEAL Evaluator semantics NEXUS
relies on (scale bookkeeping, level dropping, NAF rotations) and NEXUS's own
operators from src/ckks_evaluator.cpp, src/gelu.cpp, src/softmax.cpp and
src/layer_norm.cpp, on top of the C oracle (nexus_oracle.c).  Given the same
keys and input ciphertext they produce SEAL's output words; the tests check
that against the real NEXUS-on-SEAL build where it exists, and check the CUDA
engine against this restatement everywhere.
"""
from __future__ import annotations

import math

import numpy as np

from . import pyoracle as po


class Ct:
    """Ciphertext: data [size][limbs][N] (NTT form) and its scale."""

    def __init__(self, data: np.ndarray, scale: float):
        self.data = np.ascontiguousarray(data, dtype=np.uint64)
        self.scale = float(scale)

    @property
    def limbs(self):
        return self.data.shape[1]

    def copy(self):
        return Ct(self.data.copy(), self.scale)


class Pt:
    """Plaintext: a vector encode ([limbs][N], NTT form) or a scalar encode
    (one residue per limb: SEAL's scalar plaintext holds it in every slot)."""

    def __init__(self, scale: float, data: np.ndarray | None = None, per_limb: np.ndarray | None = None):
        self.scale = float(scale)
        self.data = data
        self.per_limb = per_limb

    @property
    def limbs(self):
        return self.data.shape[0] if self.data is not None else len(self.per_limb)

    def copy(self):
        return Pt(self.scale, None if self.data is None else self.data.copy(),
                  None if self.per_limb is None else self.per_limb.copy())


def are_close(a: float, b: float) -> bool:
    """util::are_close (util/common.h:569-573)."""
    sf = max(abs(a), abs(b), 1.0)
    return abs(a - b) < np.finfo(np.float64).eps * sf


def naf(value: int) -> list[int]:
    """util::naf (util/numth.h:22-42)."""
    res = []
    sign = value < 0
    value = abs(value)
    i = 0
    while value:
        zi = (2 - (value & 3)) if (value & 1) else 0
        value = (value - zi) >> 1
        if zi:
            res.append((-zi if sign else zi) * (1 << i))
        i += 1
    return res


class Evaluator:
    """SEAL's Evaluator/CKKSEncoder semantics over the oracle primitives.

    Levels are identified by their number of data limbs (SEAL's parms_id)."""

    def __init__(self, oc: po.OracleContext, relin_key=None, galois_keys: dict | None = None):
        self.oc = oc
        self.n = oc.n
        self.slots = oc.n // 2
        self.top = oc.k - 1
        self.q = oc.moduli
        self.relin_key = relin_key
        self.galois_keys = galois_keys or {}
        self._bits = {}

    # ---- helpers -----------------------------------------------------------
    def total_bits(self, limbs):
        if limbs not in self._bits:
            p = 1
            for q in self.q[:limbs]:
                p *= q
            self._bits[limbs] = p.bit_length()
        return self._bits[limbs]

    def _check_scale(self, scale, limbs):
        # is_scale_within_bounds (evaluator.cpp:29-47)
        if scale <= 0 or int(math.log2(scale)) >= self.total_bits(limbs):
            raise ValueError("scale out of bounds")

    # ---- encoding (CKKSEncoder) -------------------------------------------
    def encode(self, values, scale, limbs=None):
        limbs = limbs or self.top
        return Pt(scale, data=self.oc.encode(values, scale, limbs))

    def encode_scalar(self, value, scale, limbs=None):
        limbs = limbs or self.top
        return Pt(scale, per_limb=self.oc.encode_scalar(value, scale, limbs))

    def encode_then_drop(self, values, scale, limbs):
        """SEAL's encode(values, scale) at the top level, then mod_switch_to(limbs)."""
        if np.ndim(values) == 0:
            return Pt(scale, per_limb=self.oc.encode_scalar(float(values), scale, self.top)[:limbs].copy())
        return Pt(scale, data=np.ascontiguousarray(self.oc.encode(values, scale, self.top)[:limbs]))

    # ---- fork ops (evaluator.cpp:395-590 of the bootstrapping SEAL) ----------
    def add_const(self, ct, value):
        return self.add_plain(ct, self.encode_then_drop(value, ct.scale, ct.limbs))

    def multiply_const(self, ct, value):
        return self.multiply_plain(ct, self.encode_then_drop(value, ct.scale, ct.limbs))

    def multiply_vector_reduced_error(self, ct, values):
        return self.multiply_plain(ct, self.encode_then_drop(np.asarray(values), ct.scale, ct.limbs))

    def _adjust_down(self, hi, lo):
        q_top = float(self.q[hi.limbs - 1])
        scale_adjust = lo.scale * q_top / (hi.scale * hi.scale)
        adj = self.multiply_const(hi, scale_adjust)
        adj.scale = lo.scale * q_top
        adj = self.rescale(adj)
        return self.mod_switch_to(adj, lo.limbs)

    def _reduced(self, a, b, op):
        a = a.copy()
        if a.limbs == b.limbs:
            a.scale = b.scale
            return op(a, b)
        if a.limbs < b.limbs:
            adj = self._adjust_down(b, a)
            a.scale = adj.scale
            return op(a, adj)
        adj = self._adjust_down(a, b)
        adj.scale = b.scale
        return op(adj, b)

    def add_reduced_error(self, a, b):
        return self._reduced(a, b, self.add)

    def sub_reduced_error(self, a, b):
        return self._reduced(a, b, self.sub)

    def multiply_reduced_error(self, a, b):
        """multiply_inplace_reduced_error: level matching, multiply, relinearize."""
        return self.relinearize(self._reduced(a, b, self.multiply))

    # ---- level management ------------------------------------------------------
    def mod_switch_to(self, x, limbs):
        """mod_switch_to_inplace (evaluator.cpp:1630): drop limbs, keep scale."""
        if limbs > x.limbs:
            raise ValueError("cannot switch to higher level modulus")
        if isinstance(x, Ct):
            return Ct(x.data[:, :limbs], x.scale)
        if x.data is not None:
            return Pt(x.scale, data=np.ascontiguousarray(x.data[:limbs]))
        return Pt(x.scale, per_limb=x.per_limb[:limbs].copy())

    def mod_switch_to_next(self, x):
        return self.mod_switch_to(x, x.limbs - 1)

    def rescale(self, ct: Ct) -> Ct:
        """rescale_to_next (evaluator.cpp:1402-1480)."""
        if ct.limbs < 2:
            raise ValueError("end of modulus switching chain reached")
        scale = ct.scale / float(self.q[ct.limbs - 1])
        self._check_scale(scale, ct.limbs - 1)
        return Ct(self.oc.rescale(ct.data), scale)

    # ---- arithmetic ---------------------------------------------------------------
    def _same_level(self, a, b):
        if a.limbs != b.limbs:
            raise ValueError("encrypted1 and encrypted2 parameter mismatch")

    def multiply(self, a: Ct, b: Ct) -> Ct:
        self._same_level(a, b)
        scale = a.scale * b.scale
        self._check_scale(scale, a.limbs)
        return Ct(self.oc.multiply(a.data, b.data), scale)

    def square(self, a: Ct) -> Ct:
        return self.multiply(a, a)

    def relinearize(self, ct: Ct) -> Ct:
        if ct.data.shape[0] == 2:
            return ct.copy()
        return Ct(self.oc.relinearize(ct.data, self.relin_key), ct.scale)

    def add(self, a: Ct, b: Ct) -> Ct:
        self._same_level(a, b)
        if not are_close(a.scale, b.scale):
            raise ValueError("scale mismatch")
        return Ct(self.oc.add(a.data, b.data), a.scale)

    def sub(self, a: Ct, b: Ct) -> Ct:
        self._same_level(a, b)
        if not are_close(a.scale, b.scale):
            raise ValueError("scale mismatch")
        return Ct(self.oc.sub(a.data, b.data), a.scale)

    def negate(self, a: Ct) -> Ct:
        q = np.array(self.q[:a.limbs], dtype=np.uint64).reshape(1, -1, 1)
        return Ct(np.where(a.data == 0, np.uint64(0), q - a.data), a.scale)

    def _plain_arith(self, ct: Ct, pt: Pt, sub: bool) -> Ct:
        if ct.limbs != pt.limbs:
            raise ValueError("encrypted and plain parameter mismatch")
        if not are_close(ct.scale, pt.scale):
            raise ValueError("scale mismatch")
        out = ct.data.copy()
        if pt.data is not None:
            fn = self.oc.sub if sub else self.oc.add
            out[0] = fn(ct.data[0:1], pt.data[None])[0]
        else:
            out[0] = self.oc.add_scalar(ct.data[0], pt.per_limb, sub=sub)
        return Ct(out, ct.scale)

    def add_plain(self, ct: Ct, pt: Pt) -> Ct:
        return self._plain_arith(ct, pt, False)

    def sub_plain(self, ct: Ct, pt: Pt) -> Ct:
        return self._plain_arith(ct, pt, True)

    def multiply_plain(self, ct: Ct, pt: Pt) -> Ct:
        """multiply_plain_ntt (evaluator.cpp:2336-2373)."""
        if ct.limbs != pt.limbs:
            raise ValueError("encrypted and plain parameter mismatch")
        scale = ct.scale * pt.scale
        self._check_scale(scale, ct.limbs)
        if pt.data is not None:
            data = self.oc.multiply_plain(ct.data, pt.data)
        else:
            data = self.oc.multiply_scalar(ct.data, pt.per_limb)
        return Ct(data, scale)

    # ---- rotations -------------------------------------------------------------------
    def apply_galois(self, ct: Ct, elt: int) -> Ct:
        if elt not in self.galois_keys:
            raise ValueError("Galois key not present")
        return Ct(self.oc.apply_galois(ct.data, elt, self.galois_keys[elt]), ct.scale)

    def rotate(self, ct: Ct, steps: int) -> Ct:
        """rotate_internal with its NAF fallback (evaluator.cpp:2667-2722)."""
        if steps == 0:
            return ct.copy()
        elt = po.galois_elt_from_step(self.oc.log_n, steps)
        if elt in self.galois_keys:
            return self.apply_galois(ct, elt)
        parts = naf(steps)
        if len(parts) == 1:
            raise ValueError("Galois key not present")
        out = ct
        for st in parts:
            if abs(st) != (self.n >> 1):
                out = self.rotate(out, st)
        return out

    def conjugate(self, ct: Ct) -> Ct:
        return self.apply_galois(ct, po.galois_elt_from_step(self.oc.log_n, 0))


class CKKSEvaluator:
    """NEXUS's CKKSEvaluator (src/ckks_evaluator.{h,cpp}) on the oracle."""

    # constants of src/ckks_evaluator.h:14-27
    F4_COEFFS = [0, 315, 0, -420, 0, 378, 0, -180, 0, 35]
    F4_SCALE = 1 << 7
    G4_COEFFS = [0, 5850, 0, -34974, 0, 97015, 0, -113492, 0, 46623]
    G4_SCALE = 1 << 10

    def __init__(self, ev: Evaluator, scale: float):
        self.ev = ev
        self.scale = float(scale)
        self.slot_count = ev.slots

    def init_vec_with_value(self, n, value):
        return np.full(n, float(value))

    def get_modulus(self, x: Ct, k: int) -> int:
        """modulus[size - k] of x's level (src/ckks_evaluator.cpp:511-515)."""
        if x.limbs - k < 0:
            raise ValueError("level too low for the degree-9 evaluation")
        return self.ev.q[x.limbs - k]

    # src/ckks_evaluator.cpp:181-212
    def sgn_eval(self, x: Ct, d_g: int, d_f: int, sgn_factor: float = 0.5) -> Ct:
        f4 = [c / self.F4_SCALE for c in self.F4_COEFFS]
        g4 = [c / self.G4_SCALE for c in self.G4_COEFFS]
        f4_last = [c * sgn_factor for c in f4]
        g4_last = [c * sgn_factor for c in g4]
        dest = x
        for i in range(d_g):
            dest = self.eval_odd_deg9_poly(g4_last if i == d_g - 1 else g4, dest)
        for i in range(d_f):
            dest = self.eval_odd_deg9_poly(f4_last if i == d_f - 1 else f4, dest)
        return dest

    # src/ckks_evaluator.cpp:214-364
    def eval_odd_deg9_poly(self, a, x: Ct) -> Ct:
        ev = self.ev
        D = x.scale
        p = self.get_modulus(x, 2)
        q = self.get_modulus(x, 3)
        r = self.get_modulus(x, 4)
        x2 = ev.rescale(ev.relinearize(ev.square(x)))
        x = ev.mod_switch_to_next(x)
        x3 = ev.rescale(ev.relinearize(ev.multiply(x2, x)))
        x6 = ev.rescale(ev.relinearize(ev.square(x3)))
        # T1
        a5_scale = D / x2.scale * p / x3.scale * q
        T1 = ev.rescale(ev.multiply_plain(x2, ev.encode_scalar(a[5], a5_scale, x2.limbs)))
        T1 = ev.add_plain(T1, ev.encode_scalar(a[3], T1.scale, T1.limbs))
        T1 = ev.rescale(ev.relinearize(ev.multiply(T1, x3)))
        # T2
        a9_scale = D / x3.scale * r / x6.scale * q
        T2 = ev.rescale(ev.multiply_plain(x3, ev.encode_scalar(a[9], a9_scale, x3.limbs)))
        a7_scale = T2.scale / x.scale * p
        a7x = ev.rescale(ev.multiply_plain(x, ev.encode_scalar(a[7], a7_scale, x.limbs)))
        a7x = ev.mod_switch_to(a7x, T2.limbs)
        mid = (T2.scale + a7x.scale) / 2
        T2.scale = a7x.scale = mid
        T2 = ev.add(T2, a7x)
        T2 = ev.rescale(ev.relinearize(ev.multiply(T2, x6)))
        # T3
        T3 = ev.rescale(ev.multiply_plain(x, ev.encode_scalar(a[1], float(p), x.limbs)))
        mid3 = (T1.scale + T2.scale + T3.scale) / 3
        T1.scale = T2.scale = T3.scale = mid3
        dest = T2
        dest = ev.add(dest, ev.mod_switch_to(T1, dest.limbs))
        dest = ev.add(dest, ev.mod_switch_to(T3, dest.limbs))
        return dest

    # src/ckks_evaluator.cpp:366-422
    def newtonIter(self, x: Ct, res: Ct, iters: int = 4) -> Ct:
        ev = self.ev
        for _ in range(iters):
            three_half = ev.encode_scalar(1.5, self.scale)
            neg_half = ev.encode_scalar(-0.5, self.scale)
            res_sq = ev.rescale(ev.relinearize(ev.square(res)))
            res_x = ev.rescale(ev.multiply_plain(x, ev.mod_switch_to(neg_half, x.limbs)))
            if res.limbs < res_x.limbs:  # chain_index(res) < chain_index(res_x)
                res_x = ev.mod_switch_to(res_x, res.limbs)
            else:
                res = ev.mod_switch_to(res, res_x.limbs)
            res_x = ev.rescale(ev.relinearize(ev.multiply(res_x, res)))
            res_sq = ev.mod_switch_to(res_sq, res_x.limbs)
            res_x = ev.rescale(ev.relinearize(ev.multiply(res_x, res_sq)))
            res = ev.rescale(ev.multiply_plain(res, ev.mod_switch_to(three_half, res.limbs)))
            res = ev.mod_switch_to(res, res_x.limbs)
            res_x.scale = self.scale
            res.scale = self.scale
            res = ev.add(res, res_x)
        return res

    # src/ckks_evaluator.cpp:424-478
    def goldSchmidtIter(self, v: Ct, y: Ct, d: int = 1):
        ev = self.ev
        constant = ev.encode_scalar(0.5, self.scale)
        v = ev.mod_switch_to(v, y.limbs)
        x = ev.rescale(ev.relinearize(ev.multiply(v, y)))
        h = ev.rescale(ev.multiply_plain(y, ev.mod_switch_to(constant, y.limbs)))
        for _ in range(d):
            constant = ev.encode_scalar(0.5, self.scale)
            r = ev.rescale(ev.relinearize(ev.multiply(x, h)))
            r.scale = self.scale
            temp = ev.negate(r)
            r = ev.add_plain(temp, ev.mod_switch_to(constant, temp.limbs))
            x = ev.mod_switch_to(x, r.limbs)
            temp = ev.rescale(ev.relinearize(ev.multiply(x, r)))
            x.scale = self.scale
            temp.scale = self.scale
            x = ev.add(ev.mod_switch_to(x, temp.limbs), temp)
            h = ev.mod_switch_to(h, r.limbs)
            temp = ev.rescale(ev.relinearize(ev.multiply(h, r)))
            h.scale = self.scale
            temp.scale = self.scale
            h = ev.add(ev.mod_switch_to(h, temp.limbs), temp)
        constant = ev.encode_scalar(2.0, self.scale)
        h = ev.rescale(ev.multiply_plain(h, ev.mod_switch_to(constant, h.limbs)))
        return x, h

    # src/ckks_evaluator.cpp:480-485
    def invert_sqrt(self, x: Ct, d_newt: int = 5, d_gold: int = 2) -> Ct:
        res = self.initGuess(x)
        y = self.newtonIter(x, res, d_newt)
        return self.goldSchmidtIter(x, y, d_gold)[1]

    # src/ckks_evaluator.cpp:487-509
    def inverse(self, x: Ct, iters: int = 4) -> Ct:
        ev = self.ev
        one = ev.encode_scalar(1.0, x.scale, x.limbs)
        y = ev.negate(ev.sub_plain(x, one))
        tmp = ev.add_plain(y, one)
        res = tmp
        for _ in range(iters):
            y = ev.rescale(ev.relinearize(ev.square(y)))
            one = ev.encode_scalar(1.0, y.scale, y.limbs)
            tmp = ev.add_plain(y, one)
            res = ev.mod_switch_to(res, tmp.limbs)
            res = ev.rescale(ev.relinearize(ev.multiply(res, tmp)))
        return res

    # src/ckks_evaluator.cpp:517-532
    def initGuess(self, x: Ct) -> Ct:
        A = self.ev.encode_scalar(-1.29054537e-04, self.scale)
        B = self.ev.encode_scalar(1.29054537e-01, self.scale)
        return self.evalLine(x, A, B)

    def evalLine(self, x: Ct, m: Pt, c: Pt) -> Ct:
        ev = self.ev
        x = ev.rescale(ev.multiply_plain(x, ev.mod_switch_to(m, x.limbs)))
        c = ev.mod_switch_to(c, x.limbs)
        x.scale = self.scale
        return ev.add_plain(x, c)

    # src/ckks_evaluator.cpp:534-548
    def exp(self, x: Ct) -> Ct:
        ev = self.ev
        x = ev.rescale(ev.multiply_plain(x, ev.encode_scalar(0.0078125, x.scale, x.limbs)))
        x = ev.add_plain(x, ev.encode_scalar(1.0, x.scale, x.limbs))
        for _ in range(7):
            x = ev.rescale(ev.relinearize(ev.square(x)))
        return x


def gelu(ck: CKKSEvaluator, x: Ct) -> Ct:
    """GeLUEvaluator::gelu (src/gelu.cpp:5-111)."""
    ev = ck.ev
    sc = ck.slot_count
    p0 = ev.encode(ck.init_vec_with_value(sc, -3.5), x.scale, x.limbs)
    p1 = ev.encode(ck.init_vec_with_value(sc, 3.5), x.scale, x.limbs)
    delta = ev.encode(ck.init_vec_with_value(sc, 1.0 / 8.5), x.scale, x.limbs)
    b0 = ev.rescale(ev.multiply_plain(ev.sub_plain(x, p0), delta))
    b1 = ev.rescale(ev.multiply_plain(ev.sub_plain(x, p1), delta))
    b0 = ck.sgn_eval(b0, 2, 2)
    b1 = ck.sgn_eval(b1, 2, 2)
    zpf = ev.encode(ck.init_vec_with_value(sc, 0.5), b1.scale, b1.limbs)
    a1 = ev.sub(b0, b1)
    a2 = ev.add_plain(b1, zpf)
    x_2 = ev.rescale(ev.relinearize(ev.square(x)))
    x_4 = ev.rescale(ev.relinearize(ev.square(x_2)))
    x_2 = ev.mod_switch_to(x_2, x_4.limbs)
    x_6 = ev.rescale(ev.relinearize(ev.multiply(x_2, x_4)))
    x_8 = ev.rescale(ev.relinearize(ev.square(x_4)))
    x_2 = ev.mod_switch_to(x_2, x_8.limbs)
    x_10 = ev.rescale(ev.relinearize(ev.multiply(x_2, x_8)))
    x_12 = ev.rescale(ev.relinearize(ev.square(x_6)))
    A = [2.25775755e-04, 0.5, 3.96880960e-01, -6.37042698e-02, 8.38841647e-03, -7.17830961e-04,
         3.49617829e-05, -7.26059653e-07]
    coeff = [ev.encode_scalar(a, ck.scale) for a in A]
    cts = [None, x, x_2, x_4, x_6, x_8, x_10, x_12]
    for i in range(1, 8):
        coeff[i] = ev.mod_switch_to(coeff[i], cts[i].limbs)
        cts[i] = ev.rescale(ev.multiply_plain(cts[i], coeff[i]))
        cts[i].scale = ck.scale
    Ax = cts[7]
    for i in range(1, 7):
        Ax = ev.add(Ax, ev.mod_switch_to(cts[i], Ax.limbs))
    Ax = ev.add_plain(Ax, ev.mod_switch_to(coeff[0], Ax.limbs))
    Ax = ev.mod_switch_to(Ax, a1.limbs)
    s1 = ev.rescale(ev.relinearize(ev.multiply(Ax, a1)))
    xx = ev.mod_switch_to(x, a2.limbs)
    s2 = ev.rescale(ev.relinearize(ev.multiply(xx, a2)))
    s1.scale = ck.scale
    s2.scale = ck.scale
    s2 = ev.mod_switch_to(s2, s1.limbs)
    return ev.add(s1, s2)


def softmax(ck: CKKSEvaluator, x: Ct, length: int) -> Ct:
    """SoftmaxEvaluator::softmax (src/softmax.cpp:6-42)."""
    ev = ck.ev
    log_step = int(math.log2(length))
    tmp = ev.rotate(x, -length)
    x = ev.add(x, tmp)
    exp_x = ck.exp(x)
    tmp = exp_x
    res = None
    for i in range(log_step):
        res = ev.rotate(tmp, 2 ** i)
        res = ev.add(res, tmp)
        tmp = res
    res = ev.rescale(ev.multiply_plain(res, ev.encode_scalar(0.01, res.scale, res.limbs)))
    res = ck.inverse(res)
    res = ev.rescale(ev.multiply_plain(res, ev.encode_scalar(0.01, res.scale, res.limbs)))
    exp_x = ev.mod_switch_to(exp_x, res.limbs)
    return ev.rescale(ev.relinearize(ev.multiply(res, exp_x)))


def layer_norm(ck: CKKSEvaluator, x: Ct, length: int) -> Ct:
    """LNEvaluator::layer_norm (src/layer_norm.cpp:6-33)."""
    ev = ck.ev
    log_step = int(math.log2(length))
    tmp = ev.rotate(x, -length)
    x = ev.add(x, tmp)
    x2 = ev.rescale(ev.relinearize(ev.square(x)))
    tmp = x2
    res = None
    for i in range(log_step):
        res = ev.rotate(tmp, 2 ** i)
        res = ev.add(res, tmp)
        tmp = res
    res = ev.rescale(ev.multiply_plain(res, ev.encode_scalar(1.0 / 768, res.scale, res.limbs)))
    res = ck.invert_sqrt(res, 4, 2)
    x = ev.mod_switch_to(x, res.limbs)
    return ev.rescale(ev.relinearize(ev.multiply(res, x)))


def argmax(ck: CKKSEvaluator, bs, x: Ct, length: int) -> Ct:
    """ArgmaxEvaluator::argmax (src/argmax.cpp:9-81); bs is an
    oracle.bootstrap.Bootstrapper over the same evaluator."""
    ev = ck.ev
    log_step = int(math.log2(length))
    x = ev.add(x, ev.rotate(x, -length))
    a = x
    for i in range(log_step):
        b = ev.rotate(a, 1 << i)
        a_plus_b = ev.add(a, b)
        a_minus_b = ev.sub(a, b)
        sign = ck.sgn_eval(a_minus_b, 2, 2)
        a_minus_b = ev.mod_switch_to(a_minus_b, sign.limbs)
        a_minus_b_sgn = ev.rescale(ev.relinearize(ev.multiply(a_minus_b, sign)))
        half = ev.encode_scalar(0.5, a_plus_b.scale, a_plus_b.limbs)
        a_plus_b = ev.rescale(ev.multiply_plain(a_plus_b, half))
        a_plus_b.scale = a_minus_b_sgn.scale
        a_plus_b = ev.mod_switch_to(a_plus_b, a_minus_b_sgn.limbs)
        a = ev.add(a_plus_b, a_minus_b_sgn)
        # ArgmaxEvaluator::bootstrap (:83-106)
        a = ev.mod_switch_to(a, 1)
        bs.final_scale = a.scale
        a = bs.bootstrap_3(a)
    x.scale = a.scale
    x = ev.mod_switch_to(x, a.limbs)
    res = ck.sgn_eval(ev.sub(x, a), 2, 2, 1.0)
    return ev.add_plain(res, ev.encode_scalar(1.0, res.scale, res.limbs))


def negacyclic_shift(coeffs: np.ndarray, index: int, q_per_limb) -> np.ndarray:
    """negacyclic_shift_poly_coeffmod (util/polyarithsmallmod.cpp:319-370) on
    coefficient-form residues [..., limbs, N]: multiply by X^index mod X^N+1."""
    n = coeffs.shape[-1]
    out = np.empty_like(coeffs)
    raw = np.arange(n, dtype=np.int64) + index
    dst = raw & (n - 1)
    neg = (raw & n) != 0
    q = np.array(q_per_limb, dtype=np.uint64).reshape((-1, 1))
    val = np.where(neg & (coeffs != 0), q - coeffs, coeffs)
    out[..., dst] = val
    return out


class MMEvaluator:
    """NEXUS's MMEvaluator (src/matrix_mul.cpp) on the oracle: the ciphertext
    expansion tree and the ct x pt accumulation, generalised from the
    hard-coded 768 x 64 shape to R x K."""

    def __init__(self, ck: CKKSEvaluator):
        self.ck = ck
        self.ev = ck.ev
        n = self.ev.n
        # ckks->rots (src/ckks_evaluator.h:83-85): Galois elements (N + 2^i) / 2^i
        self.rots = [(n + 2 ** i) // 2 ** i for i in range(int(math.ceil(math.log2(n))))]

    # src/matrix_mul.cpp:131-172
    def multiply_power_of_x(self, ct: Ct, index: int) -> Ct:
        oc = self.ev.oc
        limbs = ct.limbs
        coeffs = oc.ntt(ct.data, 0, limbs, inverse=True)
        shifted = negacyclic_shift(coeffs, index, self.ev.q[:limbs])
        return Ct(oc.ntt(shifted, 0, limbs), ct.scale)

    # src/matrix_mul.cpp:101-129
    def expand_ciphertext(self, ct: Ct, m: int) -> list:
        ev = self.ev
        n = ev.n
        logm = int(math.ceil(math.log2(m)))
        temp = [ct]
        for i in range(logm):
            newtemp = [None] * (2 * len(temp))
            index_raw = (n << 1) - (1 << i)
            index = (index_raw * self.rots[i]) % (n << 1)
            for a in range(len(temp)):
                rotated = ev.apply_galois(temp[a], self.rots[i])
                newtemp[a] = ev.add(temp[a], rotated)
                shifted = self.multiply_power_of_x(temp[a], index_raw)
                rshift = self.multiply_power_of_x(rotated, index)
                newtemp[a + len(temp)] = ev.add(shifted, rshift)
            temp = newtemp
        return temp

    # src/matrix_mul.cpp:174-246 after the expansion: output r = sum_k leaf[r*K+k] * pts[k],
    # scale times the expansion factor, rescaled down to one prime
    def accumulate(self, leaves: list, pts: list, rows: int, cols: int, factor: float) -> list:
        ev = self.ev
        res = []
        for r in range(rows):
            terms = [ev.multiply_plain(leaves[r * cols + k], pts[k]) for k in range(cols)]
            acc = terms[0]
            for t in terms[1:]:
                acc = ev.add(acc, t)
            acc.scale *= factor
            while acc.limbs > 1:
                acc = ev.rescale(acc)
            res.append(acc)
        return res
