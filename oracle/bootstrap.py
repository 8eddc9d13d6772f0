"""CPU restatement of NEXUS's CKKS bootstrapping -- TEST INFRASTRUCTURE.

Follows src/bootstrapping/Bootstrapper.cpp (the three-level BSGS "_3"
bootstrap), ModularReducer.cpp and common/{Polynomial,func}.cpp call by call
on top of the SEAL-semantics evaluator of nexus_l3.py, so that given the
same keys, input ciphertext and EvalMod table it produces the words the
reference would.  The reference cannot be built here (it needs NTL), so this
restatement is pinned by (a) its evaluator ops, which are pinned to SEAL,
(b) the decrypted result matching the input, and (c) the LT diagonals being
recomputed with the reference's exact FP64 operation order.

Complex products are spelled out on real arrays, (ac - bd, ad + bc), each
product and sum rounded once, which is what std::complex<double> multiplies
to without FMA contraction.
"""
from __future__ import annotations

import math

import numpy as np

from . import nexus_l3 as l3
from . import pyoracle as po


# --------------------------------------------------------------------------
# common/func.cpp
# --------------------------------------------------------------------------

def giantstep(m: int) -> int:
    """giantstep (func.cpp:204-214): k minimising ceil(m/k) + k - 1."""
    minval, mink = m, 1
    k = 1
    while k <= 3 * math.sqrt(m):
        cur = math.ceil(m / k) + k - 1
        if cur < minval:
            minval, mink = cur, k
        k += 1
    return mink


def rotation(logslot: int, nh: int, shift: int, re: np.ndarray, im: np.ndarray):
    """rotation (func.cpp:216-225): vec rotated left by shift within each
    2^logslot block, repeated to Nh entries."""
    slotlen = 1 << logslot
    idx = slotlen + np.arange(slotlen) + shift
    assert idx.min() >= 0, "negative index (undefined in the reference)"
    idx %= slotlen
    rep = nh // slotlen
    return np.tile(re[idx], rep), np.tile(im[idx], rep)


def _cmul(ar, ai, br, bi):
    return ar * br - ai * bi, ar * bi + ai * br


# --------------------------------------------------------------------------
# LT coefficients (Bootstrapper.cpp:522-602, 1144-1954)
# --------------------------------------------------------------------------

def gen_orig_coeff(logn: int):
    """genorigcoeff for one slot count: (orig, orig_inv), each [logn][3] pairs of
    (re, im) arrays of length n."""
    n = 1 << logn
    orig = [[None] * 3 for _ in range(logn)]
    theta0 = math.pi / (2 * n)
    blocklen, blockcount = 1, n
    for i in range(logn):
        blocklen <<= 1
        blockcount >>= 1
        theta = theta0 * (1 << (logn - 1 - i))
        r = [np.zeros(n) for _ in range(3)]
        m = [np.zeros(n) for _ in range(3)]
        power = 1
        half = blocklen // 2
        for j in range(half):
            zr, zi = math.cos(theta * power), math.sin(theta * power)
            lo = np.arange(blockcount) * blocklen + j
            hi = lo + half
            r[1][lo], m[1][lo] = 1.0, 0.0
            r[1][hi], m[1][hi] = -zr, -zi
            r[0][lo], m[0][lo] = 0.0, 0.0
            r[0][hi], m[0][hi] = 1.0, 0.0
            r[2][lo], m[2][lo] = zr, zi
            r[2][hi], m[2][hi] = 0.0, 0.0
            power = (5 * power) % (1 << (i + 3))
        orig[i] = [(r[t], m[t]) for t in range(3)]

    inv = [[None] * 3 for _ in range(logn)]
    theta0 = -math.pi / (2 * n)
    blocklen, blockcount = n, 1
    for i in range(logn):
        theta = theta0 * (1 << i)
        r = [np.zeros(n) for _ in range(3)]
        m = [np.zeros(n) for _ in range(3)]
        power = 1
        half = blocklen // 2
        for j in range(half):
            zr, zi = math.cos(theta * power), math.sin(theta * power)
            lo = np.arange(blockcount) * blocklen + j
            hi = lo + half
            r[1][lo], m[1][lo] = 0.5, 0.0
            r[1][hi], m[1][hi] = -0.5 * zr, -0.5 * zi
            r[0][lo], m[0][lo] = 0.0, 0.0
            r[0][hi], m[0][hi] = 0.5 * zr, 0.5 * zi
            r[2][lo], m[2][lo] = 0.5, 0.0
            r[2][hi], m[2][hi] = 0.0, 0.0
            power = (5 * power) % (1 << ((logn - 1 - i) + 3))
        inv[i] = [(r[t], m[t]) for t in range(3)]
        blocklen >>= 1
        blockcount <<= 1
    return orig, inv


def _merge_level(orig, offset: int, d: int, basicstep: int, n: int, reverse_bits: bool, nslots: int, index_of):
    """One level of genfftcoeff_3 / geninvfftcoeff_3: sum over the 3^d paths of
    the products of d butterfly diagonals, accumulated in path order."""
    acc_r = [np.zeros(n) for _ in range(nslots)]
    acc_i = [np.zeros(n) for _ in range(nslots)]
    k = np.arange(n)
    for j in range(3 ** d):
        ind, pos, cnt = j, 0, []
        for p in range(d):
            res = ind % 3
            w = 1 << ((d - 1 - p) if reverse_bits else p)
            pos += (res - 1) * w
            cnt.append(res)
            ind = (ind - res) // 3
        cur = pos
        tr, ti = np.ones(n), np.zeros(n)
        for p in range(d):
            w = 1 << ((d - 1 - p) if reverse_bits else p)
            cur -= (cnt[p] - 1) * w
            idx = (k + basicstep * (n + cur)) % n
            br, bi = orig[p + offset][cnt[p]]
            tr, ti = _cmul(tr, ti, br[idx], bi[idx])
        s = index_of(pos)
        acc_r[s] = acc_r[s] + tr
        acc_i[s] = acc_i[s] + ti
    return list(zip(acc_r, acc_i))


def split3_fwd(logn: int):
    d3 = logn // 3
    d2 = (logn - d3) // 2
    d1 = logn - d3 - d2
    return d1, d2, d3


def split3_inv(logn: int):
    d1 = logn // 3
    d2 = (logn - d1) // 2
    d3 = logn - d1 - d2
    return d1, d2, d3


def gen_fft_coeff_3_full(logn: int, orig):
    """genfftcoeff_3, full-slot branch (Bootstrapper.cpp:1159-1282)."""
    n = 1 << logn
    d1, d2, d3 = split3_fwd(logn)
    t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
    c1 = _merge_level(orig, 0, d1, 1, n, False, 2 * t1 + 1, lambda pos: pos + t1)
    c2 = _merge_level(orig, d1, d2, 1 << d1, n, False, 2 * t2 + 1, lambda pos: pos + t2)
    c3 = _merge_level(orig, d1 + d2, d3, 1 << (d1 + d2), n, False, t3 + 1,
                      lambda pos: (pos + t3 + 1) % (t3 + 1))
    return c1, c2, c3


def gen_invfft_coeff_3_full(logn: int, inv, boundary_k: int):
    """geninvfftcoeff_3, full-slot branch (Bootstrapper.cpp:1567-1689)."""
    n = 1 << logn
    d1, d2, d3 = split3_inv(logn)
    t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
    c1 = _merge_level(inv, 0, d1, 1 << (logn - d1), n, True, t1 + 1, lambda pos: (pos + t1 + 1) % (t1 + 1))
    c2 = _merge_level(inv, d1, d2, 1 << (logn - d1 - d2), n, True, 2 * t2 + 1, lambda pos: pos + t2)
    c3 = _merge_level(inv, d1 + d2, d3, 1, n, True, 2 * t3 + 1, lambda pos: pos + t3)
    s = 1.0 / boundary_k
    c1 = [(r * s, i * s) for r, i in c1]
    c3 = [(r * 0.5, i * 0.5) for r, i in c3]
    return c1, c2, c3


def gen_fft_coeff_3_sparse(logn: int, orig):
    """genfftcoeff_3, sparse branch (Bootstrapper.cpp:1284-1428): diagonals of
    length 2n, the second half a copy (levels 1, 2) or i times the first
    half (level 3)."""
    n = 1 << logn
    d1, d2, d3 = split3_fwd(logn)
    t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
    c1 = _merge_level(orig, 0, d1, 1, n, False, 2 * t1 + 1, lambda pos: pos + t1)
    c2 = _merge_level(orig, d1, d2, 1 << d1, n, False, 2 * t2 + 1, lambda pos: pos + t2)
    c3 = _merge_level(orig, d1 + d2, d3, 1 << (d1 + d2), n, False, 2 * t3 + 1, lambda pos: pos + t3)
    c1 = [(np.concatenate([r, r]), np.concatenate([i, i])) for r, i in c1]
    c2 = [(np.concatenate([r, r]), np.concatenate([i, i])) for r, i in c2]
    # complex(0, 1) * z = (0*a - 1*b, 0*b + 1*a)
    c3 = [(np.concatenate([r, 0.0 * r - 1.0 * i]), np.concatenate([i, 0.0 * i + 1.0 * r])) for r, i in c3]
    return c1, c2, c3


def gen_invfft_coeff_3_sparse(logn: int, log_nh: int, inv, boundary_k: int):
    """geninvfftcoeff_3, sparse branch (Bootstrapper.cpp:1690-1818)."""
    n = 1 << logn
    d1, d2, d3 = split3_inv(logn)
    t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
    c1 = _merge_level(inv, 0, d1, 1 << (logn - d1), n, True, t1 + 1, lambda pos: (pos + t1 + 1) % (t1 + 1))
    c2 = _merge_level(inv, d1, d2, 1 << (logn - d1 - d2), n, True, 2 * t2 + 1, lambda pos: pos + t2)
    c3 = _merge_level(inv, d1 + d2, d3, 1, n, True, 2 * t3 + 1, lambda pos: pos + t3)
    s = 1.0 / (boundary_k * (1 << (log_nh - logn)))
    c1 = [(r * s, i * s) for r, i in c1]
    out3 = []
    for r, i in c3:
        r, i = r * 0.5, i * 0.5
        # complex(0, -1) * z = (0*a - (-1)*b, 0*b + (-1)*a)
        out3.append((np.concatenate([r, 0.0 * r - (-1.0) * i]), np.concatenate([i, 0.0 * i + (-1.0) * r])))
    return c1, c2, out3


def rot_key_steps_3(logn: int, log_nh: int) -> list[int]:
    """Rotation steps of the driver (src/bootstrapping.cpp:111-118: 0 and 2^i)
    followed by addLeftRotKeys_Linear_to_vector_3 (Bootstrapper.cpp:89-184)."""
    nh = 1 << log_nh
    steps = [0] + [1 << i for i in range(log_nh)]

    def push(v):
        if v not in steps:
            steps.append(v)

    d1 = logn // 3
    d2 = (logn - d1) // 2
    d3 = logn - d1 - d2
    t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
    bs1, bs2, bs3 = 1 << (logn - d1), 1 << (logn - d1 - d2), 1
    gs1 = giantstep(t1 + 1)
    gs1_e = giantstep(2 * t1 + 1) if logn != log_nh else 0
    gs2 = giantstep(2 * t2 + 1)
    gs3 = giantstep(2 * t3 + 1)
    start1 = -t1 + gs1 * (t1 // gs1)
    gfirst1 = -(t1 // gs1)
    glast1 = (2 * t1) // gs1 + gfirst1
    glast1_e = t1 // gs1 if logn != log_nh else 0
    start2 = -t2 + gs2 * (t2 // gs2)
    gfirst2 = -(t2 // gs2)
    glast2 = (2 * t2) // gs2 + gfirst2
    start3 = -t3 + gs3 * (t3 // gs3)
    gfirst3 = -(t3 // gs3)
    glast3 = (2 * t3) // gs3 + gfirst3
    for i in range(start1, start1 + gs1):
        if i:
            push((nh + i * bs1) % nh)
    for i in range(1, gs1_e):
        push(i * bs1)
    for i in range(start2, start2 + gs2):
        if i:
            push((nh + i * bs2) % nh)
    for i in range(start3, start3 + gs3):
        if i:
            push((nh + i * bs3) % nh)
    for i in range(gfirst1, glast1 + 1):
        if i:
            push((nh + i * gs1 * bs1) % nh)
    for i in range(1, glast1_e + 1):
        push(i * gs1_e * bs1)
    for i in range(gfirst2, glast2 + 1):
        if i:
            push((nh + i * gs2 * bs2) % nh)
    for i in range(gfirst3, glast3 + 1):
        if i:
            push((nh + i * gs3 * bs3) % nh)
    return steps


# --------------------------------------------------------------------------
# Bootstrapper
# --------------------------------------------------------------------------

class Bootstrapper:
    """Bootstrapper (Bootstrapper.h:15-221), full-slot three-level path."""

    def __init__(self, ev: l3.Evaluator, loge: int, logn: int, log_nh: int, total_level: int,
                 final_scale: float, boundary_k: int, sin_cos_deg: int, scale_factor: int,
                 inverse_deg: int, table: dict):
        self.ev = ev
        self.loge, self.logn, self.log_nh, self.L = loge, logn, log_nh, total_level
        self.n, self.nh = 1 << logn, 1 << log_nh
        self.final_scale = float(final_scale)
        self.initial_scale = None
        self.boundary_k = boundary_k
        self.sin_cos_deg = sin_cos_deg
        self.num_double_formula = scale_factor
        self.inverse_deg = inverse_deg
        if table["deg"] != sin_cos_deg or table["boundary_K"] != boundary_k or table["double_angle"] != scale_factor:
            raise ValueError("EvalMod table does not match the parameters")
        if table.get("inverse_deg", 1) != inverse_deg:
            raise ValueError("EvalMod table is for another inverse_deg")
        self.heap_k, self.heap_m = table["heap_k"], table["heap_m"]
        self.heap = table["nodes"]
        self.scale_inverse_coeff = table["scale_inverse_coeff"]
        self.inverse = table.get("inverse")
        if inverse_deg > 1 and (self.inverse is None or len(self.inverse["power"]) != inverse_deg + 1):
            raise ValueError("EvalMod table lacks the inverse-sine polynomial")
        self.fftcoeff = self.invfftcoeff = None

    # -- setup ---------------------------------------------------------------
    def generate_LT_coefficient_3(self):
        orig, inv = gen_orig_coeff(self.logn)
        if self.logn == self.log_nh:
            self.fftcoeff = gen_fft_coeff_3_full(self.logn, orig)
            self.invfftcoeff = gen_invfft_coeff_3_full(self.logn, inv, self.boundary_k)
        else:
            self.fftcoeff = gen_fft_coeff_3_sparse(self.logn, orig)
            self.invfftcoeff = gen_invfft_coeff_3_sparse(self.logn, self.log_nh, inv, self.boundary_k)

    def rotation_steps(self):
        return rot_key_steps_3(self.logn, self.log_nh)

    # -- primitives -----------------------------------------------------------
    def _rot(self, ct, step):
        return self.ev.rotate(ct, step)

    def _mul_vec(self, ct, re, im):
        return self.ev.multiply_vector_reduced_error(ct, re + 1j * im)

    def bsgs_linear_transform(self, ct, totlen, basicstep, coeff_logn, coeff):
        """Bootstrapper.cpp:1997-2062."""
        ev, nh = self.ev, self.nh
        gs = giantstep(2 * totlen + 1)
        start = -totlen + gs * (totlen // gs)
        gfirst = -(totlen // gs)
        glast = (2 * totlen) // gs + gfirst
        baby = [ct.copy() if i == 0 else self._rot(ct, (nh + i * basicstep) % nh) for i in range(start, start + gs)]
        acc = None
        for i in range(gfirst, glast + 1):
            giant = None
            jend = start + gs - 1 if i != glast else totlen - i * gs
            for j in range(start, jend + 1):
                re, im = rotation(coeff_logn, nh, -i * gs * basicstep, *coeff[i * gs + j + totlen])
                t = self._mul_vec(baby[j - start], re, im)
                giant = t if giant is None else ev.add_reduced_error(giant, t)
            if i != 0:
                giant = self._rot(giant, (nh + i * gs * basicstep) % nh)
            acc = giant if acc is None else ev.add_reduced_error(acc, giant)
        return acc

    def rotated_bsgs_linear_transform(self, ct, totlen, basicstep, coeff_logn, coeff):
        """Bootstrapper.cpp:2064-2129."""
        ev, nh = self.ev, self.nh
        gs = giantstep(totlen + 1)
        glast = totlen // gs
        baby = [ct.copy() if i == 0 else self._rot(ct, (nh + i * basicstep) % nh) for i in range(gs)]
        acc = None
        for i in range(glast + 1):
            giant = None
            jend = gs - 1 if i != glast else totlen - i * gs
            for j in range(jend + 1):
                re, im = rotation(coeff_logn, nh, -i * gs * basicstep, *coeff[i * gs + j])
                t = self._mul_vec(baby[j], re, im)
                giant = t if giant is None else ev.add_reduced_error(giant, t)
            if i != 0:
                giant = self._rot(giant, (nh + i * gs * basicstep) % nh)
            acc = giant if acc is None else ev.add_reduced_error(acc, giant)
        return acc

    def sflinv_full_3(self, ct):
        """Bootstrapper.cpp:2604-2622."""
        logn = self.logn
        d1, d2, d3 = split3_inv(logn)
        t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
        c1, c2, c3 = self.invfftcoeff
        x = self.ev.rescale(self.rotated_bsgs_linear_transform(ct, t1, 1 << (logn - d1), logn, c1))
        x = self.ev.rescale(self.bsgs_linear_transform(x, t2, 1 << (logn - d1 - d2), logn, c2))
        return self.ev.rescale(self.bsgs_linear_transform(x, t3, 1, logn, c3))

    def sfl_full_3(self, ct):
        """Bootstrapper.cpp:2458-2496."""
        logn = self.logn
        d1, d2, d3 = split3_fwd(logn)
        t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
        if t2 != t3:
            raise ValueError("sfl_full_3 needs equal second and third splits (logn % 3 != 2)")
        c1, c2, c3 = self.fftcoeff
        x = self.ev.rescale(self.bsgs_linear_transform(ct, t1, 1, logn, c1))
        x = self.ev.rescale(self.bsgs_linear_transform(x, t2, 1 << d1, logn, c2))
        mod_zero = float(self.ev.q[0])
        curr_mod = float(self.ev.q[x.limbs - 1])
        # fftcoeff3 * curr_mod * mod_zero * final_scale / (scale * scale * initial_scale), left to right
        f = [None] * (t2 + 1)
        for i in range(t2 + 1):
            re, im = c3[i]
            s = x.scale * x.scale * self.initial_scale
            f[i] = ((re * curr_mod) * mod_zero * self.final_scale / s,
                    (im * curr_mod) * mod_zero * self.final_scale / s)
        return self.ev.rescale(self.rotated_bsgs_linear_transform(x, t3, 1 << (d1 + d2), logn, f))

    def sflinv_3(self, ct):
        """Bootstrapper.cpp:2578-2602."""
        logn = self.logn
        d1, d2, d3 = split3_inv(logn)
        t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
        c1, c2, c3 = self.invfftcoeff
        x = self.ev.rescale(self.rotated_bsgs_linear_transform(ct, t1, 1 << (logn - d1), logn, c1))
        x = self.ev.rescale(self.bsgs_linear_transform(x, t2, 1 << (logn - d1 - d2), logn, c2))
        return self.ev.rescale(self.bsgs_linear_transform(x, t3, 1, logn + 1, c3))

    def sfl_3(self, ct):
        """Bootstrapper.cpp:2419-2456."""
        logn = self.logn
        d1, d2, d3 = split3_fwd(logn)
        t1, t2, t3 = (1 << d1) - 1, (1 << d2) - 1, (1 << d3) - 1
        c1, c2, c3 = self.fftcoeff
        x = self.ev.rescale(self.bsgs_linear_transform(ct, t1, 1, logn + 1, c1))
        x = self.ev.rescale(self.bsgs_linear_transform(x, t2, 1 << d1, logn + 1, c2))
        mod_zero = float(self.ev.q[0])
        curr_mod = float(self.ev.q[x.limbs - 1])
        f = []
        for re, im in c3:
            s = x.scale * x.scale * self.initial_scale
            f.append(((re * curr_mod) * mod_zero * self.final_scale / s,
                      (im * curr_mod) * mod_zero * self.final_scale / s))
        return self.ev.rescale(self.bsgs_linear_transform(x, t3, 1 << (d1 + d2), logn + 1, f))

    def coefftoslot_3(self, ct):
        """Bootstrapper.cpp:2720-2725."""
        t1 = self.sflinv_3(ct)
        return self.ev.add_reduced_error(t1, self.ev.conjugate(t1))

    def slottocoeff_3(self, ct):
        """Bootstrapper.cpp:2727-2732."""
        t1 = self.sfl_3(ct)
        return self.ev.add_reduced_error(t1, self.ev.rotate(t1, self.n))

    def coefftoslot_full_3(self, ct):
        """Bootstrapper.cpp:2741-2757: (real part, imaginary part) ciphertexts."""
        ev = self.ev
        t1 = self.sflinv_full_3(ct)
        minus_i = np.zeros(self.nh) - 1j
        pt = ev.mod_switch_to(ev.encode(minus_i, 1.0), t1.limbs)
        t2 = ev.multiply_plain(t1, pt)
        t3 = ev.conjugate(t2)
        t4 = ev.conjugate(t1)
        return ev.add_reduced_error(t1, t4), ev.add_reduced_error(t2, t3)

    def slottocoeff_full_3(self, c1, c2):
        """Bootstrapper.cpp:2759-2775."""
        ev = self.ev
        plus_i = np.zeros(self.nh) + 1j
        pt = ev.mod_switch_to(ev.encode(plus_i, 1.0), c2.limbs)
        t1 = ev.multiply_plain(c2, pt)
        t3 = ev.add_reduced_error(c1, t1)
        return self.sfl_full_3(t3)

    def modraise_inplace(self, ct):
        """Bootstrapper.cpp:2937-2991: centred lift of the q0 limb to every data prime."""
        if ct.data.shape[0] != 2:
            raise ValueError("Ciphertexts of size 2 are supported only!")
        if ct.limbs != 1:
            raise ValueError("Ciphertexts in the lowest level are supported only!")
        oc = self.ev.oc
        coeff = oc.ntt(ct.data, 0, 1, inverse=True)[:, 0, :]
        q0 = self.ev.q[0]
        top = self.ev.top
        out = np.zeros((2, top, oc.n), dtype=np.uint64)
        neg = coeff > np.uint64(q0 >> 1)
        for j in range(top):
            q = self.ev.q[j]
            v = coeff % np.uint64(q)
            minus_q0 = np.uint64(0 if j == 0 else q - q0 % q)
            w = v + minus_q0
            w = np.where(w >= np.uint64(q), w - np.uint64(q), w)
            out[:, j, :] = np.where(neg, w, v)
        return l3.Ct(oc.ntt(out, 0, top), ct.scale)

    # -- EvalMod (ModularReducer.cpp, Polynomial.cpp:255-485) -----------------
    def homomorphic_poly_evaluation(self, ct):
        return self.evaluate_heap(ct, self.heap_k, self.heap_m, self.heap)

    def evaluate_power(self, ct, coeff):
        """Polynomial::homomorphic_poly_evaluation for degree 1-3
        (Polynomial.cpp:257-325) on the power-basis coefficients."""
        ev = self.ev
        zero = 1.0 / ct.scale
        d = len(coeff) - 1
        if d == 1:
            return ev.add_const(ev.rescale(ev.multiply_const(ct, coeff[1])), coeff[0])
        squared = ev.rescale(ev.relinearize(ev.square(ct)))
        if d == 2:
            squared = ev.rescale(ev.multiply_const(squared, coeff[2]))
            if abs(coeff[1]) >= zero:
                rtn = ev.add_reduced_error(ev.rescale(ev.multiply_const(ct, coeff[1])), squared)
            else:
                rtn = squared
            return ev.add_const(rtn, coeff[0])
        if d != 3:
            raise ValueError("degree 1, 2 or 3 expected")
        cubic = ev.rescale(ev.multiply_const(ct, coeff[3]))
        cubic = ev.rescale(ev.multiply_reduced_error(cubic, squared))
        if abs(coeff[1]) >= zero:
            rtn = ev.add_reduced_error(ev.rescale(ev.multiply_const(ct, coeff[1])), cubic)
        else:
            rtn = cubic
        if abs(coeff[2]) >= zero:
            rtn = ev.add_reduced_error(rtn, ev.rescale(ev.multiply_const(squared, coeff[2])))
        return ev.add_const(rtn, coeff[0])

    def evaluate_heap(self, ct, k, m, nodes):
        ev = self.ev
        baby = [None] * k
        baby[1] = ct
        i = 2
        while i < k:
            b = ev.rescale(ev.relinearize(ev.square(baby[i // 2])))
            baby[i] = ev.add_const(ev.add(b, b), -1.0)
            i *= 2
        for i in range(1, k):
            if baby[i] is None:
                lpow2 = 1 << int(math.floor(math.log(i) / math.log(2)))
                res = i - lpow2
                diff = abs(lpow2 - res)
                b = ev.rescale(ev.multiply_reduced_error(baby[lpow2], baby[res]))
                baby[i] = ev.sub_reduced_error(ev.add(b, b), baby[diff])
        giant = [None] * m
        lpow2 = 1 << (int(math.ceil(math.log(k) / math.log(2))) - 1)
        res = k - lpow2
        diff = abs(lpow2 - res)
        if res == 0:
            giant[0] = baby[lpow2]
        elif diff == 0:
            g = ev.rescale(ev.relinearize(ev.square(baby[lpow2])))
            giant[0] = ev.add_const(ev.add(g, g), -1.0)
        else:
            g = ev.rescale(ev.multiply_reduced_error(baby[lpow2], baby[res]))
            giant[0] = ev.sub_reduced_error(ev.add(g, g), baby[diff])
        for i in range(1, m):
            g = ev.rescale(ev.relinearize(ev.square(giant[i - 1])))
            giant[i] = ev.add_const(ev.add(g, g), -1.0)

        heap = {}
        zero = 1.0 / ct.scale
        first, last = (1 << m) - 1, (1 << (m + 1)) - 1
        for i in range(first, last):
            coeffs = nodes.get(i)
            if coeffs is None:
                continue
            h = ev.rescale(ev.multiply_const(baby[1], coeffs[1]))
            if not abs(coeffs[1]) <= zero:
                h = ev.add_const(h, coeffs[0])
            for j in range(2, len(coeffs)):
                if abs(coeffs[j]) <= zero:
                    continue
                src = baby[j] if j < k else giant[0]
                t = ev.rescale(ev.multiply_const(src, coeffs[j]))
                h = ev.add_reduced_error(h, t)
            heap[i] = h
        depth, gindex = m, 0
        while depth:
            depth -= 1
            for i in range((1 << depth) - 1, (1 << (depth + 1)) - 1):
                if i not in nodes:
                    continue
                left, right = 2 * (i + 1) - 1, 2 * (i + 1)
                if left not in heap:
                    heap[i] = heap[right]
                else:
                    h = ev.rescale(ev.multiply_reduced_error(heap[left], giant[gindex]))
                    heap[i] = ev.add_reduced_error(h, heap[right])
            gindex += 1
        return heap[0]

    def modular_reduction(self, ct):
        """ModularReducer::modular_reduction (:58-78): the cosine, then the
        scaled double angles (inverse_deg == 1) or the plain double angles
        and the inverse-sine polynomial (inverse_deg > 1)."""
        ev = self.ev
        t = self.homomorphic_poly_evaluation(ct)
        if self.inverse_deg == 1:
            s = self.scale_inverse_coeff
            for _ in range(self.num_double_formula):
                s = s * s
                t = ev.rescale(ev.relinearize(ev.square(t)))
                t = ev.add_const(ev.add(t, t), -s)
            return t
        for _ in range(self.num_double_formula):
            t = ev.rescale(ev.relinearize(ev.square(t)))
            t = ev.add_const(ev.add(t, t), -1.0)
        inv = self.inverse
        if self.inverse_deg <= 3:
            return self.evaluate_power(t, inv["power"])
        return self.evaluate_heap(t, inv["heap_k"], inv["heap_m"], inv["nodes"])

    # -- API ---------------------------------------------------------------------
    def bootstrap_full_3(self, ct):
        """Bootstrapper.cpp:3224-3244."""
        x = self.modraise_inplace(ct)
        x.scale = float(self.ev.q[0])
        r1, r2 = self.coefftoslot_full_3(x)
        m1 = self.modular_reduction(r1)
        m2 = self.modular_reduction(r2)
        out = self.slottocoeff_full_3(m1, m2)
        out.scale = self.final_scale
        return out

    def bootstrap_sparse_3(self, ct):
        """Bootstrapper.cpp:3142-3222."""
        ev, nh = self.ev, self.nh
        x = self.modraise_inplace(ct)
        x.scale = float(ev.q[0])
        for i in range(self.logn, self.log_nh):
            x = ev.add(x, ev.rotate(x, 1 << i))
        if self.logn == 0:
            k = 2.0 * self.boundary_k * (1 << self.log_nh)
            v = np.array([1.0 / k if i % 2 == 0 else -1j / k for i in range(nh)])
            rtn = ev.rescale(ev.multiply_vector_reduced_error(x, v))
            rtn = ev.add_reduced_error(rtn, ev.conjugate(rtn))
        else:
            rtn = self.coefftoslot_3(x)
        mod = self.modular_reduction(rtn)
        if self.logn == 0:
            mod_zero = float(ev.q[0])
            curr_mod = float(ev.q[mod.limbs - 1])
            adj = curr_mod * mod_zero * self.final_scale / (mod.scale * mod.scale * self.initial_scale)
            v = np.array([adj if i % 2 == 0 else 1j * adj for i in range(nh)])
            out = ev.rescale(ev.multiply_vector_reduced_error(mod, v))
            out = ev.add_reduced_error(out, ev.rotate(out, 1))
        else:
            out = self.slottocoeff_3(mod)
        out.scale = self.final_scale
        return out

    def bootstrap_3(self, ct):
        """Bootstrapper.cpp:3489-3495."""
        self.initial_scale = ct.scale
        if self.logn == self.log_nh:
            return self.bootstrap_full_3(ct)
        return self.bootstrap_sparse_3(ct)


def monomial(ev: l3.Evaluator, power: int, limbs: int) -> l3.Pt:
    """The NTT form of X^power at `limbs` limbs, scale 1 (Evaluator::monomial
    of the engine): multiply_plain by it multiplies the message by X^power."""
    x = np.zeros((limbs, ev.oc.n), dtype=np.uint64)
    x[:, power] = 1
    return l3.Pt(1.0, data=ev.oc.ntt(x, 0, limbs))


def bootstrap_real_pair(bs: Bootstrapper, c0, c1):
    """Two ciphertexts of real slot values refreshed by one bootstrap_3
    (nexus_bootstrap_real_batch and the BERT layer's boot_pack): z = c0 +
    X^(N/2) c1 holds c0 + i c1, its scale doubled so that the refreshed z
    holds (c0 + i c1) / 2; then c0 = z + conj(z), c1 = (conj(z) - z) X^(N/2)."""
    ev = bs.ev
    half = ev.oc.n // 2
    z = ev.add(c0, ev.multiply_plain(c1, monomial(ev, half, 1)))
    z.scale *= 2.0
    r = bs.bootstrap_3(z)
    conj = ev.conjugate(r)
    return ev.add(r, conj), ev.multiply_plain(ev.sub(conj, r), monomial(ev, half, r.limbs))
