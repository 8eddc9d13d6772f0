"""Python handles over the NEXUS operator layer of the C ABI
(nexus_evaluator / nexus_ciphertext in include/nexus_gb300.h)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib
from .context import Context, _stream_ptr

OP_SGN_EVAL, OP_EXP, OP_INVERSE, OP_INVERT_SQRT = 0, 1, 2, 3


class Ciphertext:
    """Engine-owned ciphertext [size][limbs][N] with its scale."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib().nexus_ciphertext_create(ctx.handle, C.byref(h)), "nexus_ciphertext_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nexus_ciphertext_destroy(self._h)
            self._h = None

    @classmethod
    def from_numpy(cls, ctx: Context, data: np.ndarray, scale: float):
        ct = cls(ctx)
        a = np.ascontiguousarray(data, dtype=np.uint64)
        check(lib().nexus_ciphertext_load(ct._h, a.ctypes.data, a.shape[0], a.shape[1], float(scale), 1, None),
              "nexus_ciphertext_load")
        return ct

    @classmethod
    def from_device(cls, ctx: Context, t, scale: float, stream=None):
        ct = cls(ctx)
        check(lib().nexus_ciphertext_load(ct._h, t.data_ptr(), t.shape[0], t.shape[1], float(scale), 0,
                                          _stream_ptr(stream)), "nexus_ciphertext_load")
        return ct

    def info(self):
        size, limbs, scale, ptr = C.c_int(), C.c_int(), C.c_double(), C.c_void_p()
        check(lib().nexus_ciphertext_info(self._h, C.byref(size), C.byref(limbs), C.byref(scale), C.byref(ptr)),
              "nexus_ciphertext_info")
        return size.value, limbs.value, scale.value, ptr.value

    @property
    def scale(self):
        return self.info()[2]

    def to_numpy(self) -> np.ndarray:
        size, limbs, _, _ = self.info()
        out = np.zeros((size, limbs, self.ctx.n), dtype=np.uint64)
        check(lib().nexus_ciphertext_store(self._h, out.ctypes.data, 1, None), "nexus_ciphertext_store")
        return out

    def to_device(self):
        import torch
        size, limbs, _, _ = self.info()
        t = torch.empty((size, limbs, self.ctx.n), dtype=torch.int64, device="cuda")
        check(lib().nexus_ciphertext_store(self._h, t.data_ptr(), 0, None), "nexus_ciphertext_store")
        return t


class Evaluator:
    """NEXUS CKKSEvaluator + GELU / softmax / LayerNorm on the engine."""

    def __init__(self, ctx: Context, scale: float, relin_key=None, galois_keys: dict | None = None, stream=None):
        self.ctx = ctx
        self._keys = [relin_key] + list((galois_keys or {}).values())  # keep device tensors alive
        h = C.c_void_p()
        check(lib().nexus_evaluator_create(ctx.handle, float(scale), None if relin_key is None else
                                           relin_key.data_ptr(), _stream_ptr(stream), C.byref(h)),
              "nexus_evaluator_create")
        self._h = h
        for elt, key in (galois_keys or {}).items():
            check(lib().nexus_evaluator_add_galois_key(self._h, int(elt), key.data_ptr()),
                  "nexus_evaluator_add_galois_key")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nexus_evaluator_destroy(self._h)
            self._h = None

    def gelu(self, x: Ciphertext) -> Ciphertext:
        res = Ciphertext(self.ctx)
        check(lib().nexus_gelu(self._h, x.handle, res.handle), "nexus_gelu")
        return res

    def softmax(self, x: Ciphertext, length: int) -> Ciphertext:
        res = Ciphertext(self.ctx)
        check(lib().nexus_softmax(self._h, x.handle, int(length), res.handle), "nexus_softmax")
        return res

    def layer_norm(self, x: Ciphertext, length: int) -> Ciphertext:
        res = Ciphertext(self.ctx)
        check(lib().nexus_layer_norm(self._h, x.handle, int(length), res.handle), "nexus_layer_norm")
        return res

    def _op(self, op, x, a1=0, a2=0, f=0.0):
        res = Ciphertext(self.ctx)
        check(lib().nexus_ckks_op(self._h, op, x.handle, int(a1), int(a2), float(f), res.handle), "nexus_ckks_op")
        return res

    def sgn_eval(self, x, d_g, d_f, sgn_factor=0.5):
        return self._op(OP_SGN_EVAL, x, d_g, d_f, sgn_factor)

    def exp(self, x):
        return self._op(OP_EXP, x)

    def inverse(self, x, iters=4):
        return self._op(OP_INVERSE, x, iters)

    def invert_sqrt(self, x, d_newt=5, d_gold=2):
        return self._op(OP_INVERT_SQRT, x, d_newt, d_gold)

    # ---- MatMul (src/matrix_mul.cpp) ------------------------------------------
    def mm_power_of_x(self, x: Ciphertext, index: int) -> Ciphertext:
        res = Ciphertext(self.ctx)
        check(lib().nexus_mm_power_of_x(self._h, x.handle, int(index), res.handle), "nexus_mm_power_of_x")
        return res

    def mm_expand(self, x: Ciphertext, m: int):
        import torch
        _, limbs, _, _ = x.info()
        out = torch.empty((m, 2, limbs, self.ctx.n), dtype=torch.int64, device="cuda")
        check(lib().nexus_mm_expand(self._h, x.handle, int(m), out.data_ptr()), "nexus_mm_expand")
        return out

    def matrix_mul(self, compressed, pts, pt_scale: float, rows: int, cols: int, factor: float, bias=None):
        """compressed: list of Ciphertext; pts: CUDA int64 tensor [cols][limbs][N]; bias: slot values or None."""
        comp = (C.c_void_p * len(compressed))(*[c.handle.value for c in compressed])
        res = [Ciphertext(self.ctx) for _ in range(rows)]
        out = (C.c_void_p * rows)(*[r.handle.value for r in res])
        b = None if bias is None else np.ascontiguousarray(bias, dtype=np.float64)
        check(lib().nexus_matrix_mul(self._h, comp, len(compressed), pts.data_ptr(), float(pt_scale), int(rows),
                                     int(cols), float(factor), None if b is None else b.ctypes.data,
                                     0 if b is None else b.size, out), "nexus_matrix_mul")
        return res
