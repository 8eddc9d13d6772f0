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

    def load(self, t, scale: float, stream=None) -> None:
        """Overwrite this ciphertext with the device tensor ``t``
        [size][limbs][N] on ``stream``; a handle of at least that size keeps
        its buffer (what a captured graph's input needs)."""
        check(lib().nexus_ciphertext_load(self._h, t.data_ptr(), t.shape[0], t.shape[1], float(scale), 0,
                                          _stream_ptr(stream)), "nexus_ciphertext_load")

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

    def save_seal(self, parms_id) -> bytes:
        """SEAL's Ciphertext::save bytes (compr_mode none) for this ciphertext."""
        return seal_save(self.to_numpy(), self.scale, parms_id)

    @classmethod
    def load_seal(cls, ctx: Context, data: bytes):
        """(ciphertext, parms_id) from SEAL's Ciphertext::save bytes."""
        words, scale, pid, ntt = seal_load(data)
        if not ntt:
            raise ValueError("the engine keeps ciphertexts in NTT form")
        return cls.from_numpy(ctx, words, scale), pid

    def to_device(self):
        import torch
        size, limbs, _, _ = self.info()
        t = torch.empty((size, limbs, self.ctx.n), dtype=torch.int64, device="cuda")
        check(lib().nexus_ciphertext_store(self._h, t.data_ptr(), 0, None), "nexus_ciphertext_store")
        return t


def seal_save(words: np.ndarray, scale: float, parms_id, is_ntt_form: bool = True) -> bytes:
    """Ciphertext::save (compr_mode none) of host words [size][limbs][N]."""
    w = np.ascontiguousarray(words, dtype=np.uint64)
    size, limbs, n = w.shape
    pid = np.ascontiguousarray(parms_id, dtype=np.uint64)
    nbytes = C.c_size_t()
    log_n = n.bit_length() - 1
    u64 = C.POINTER(C.c_uint64)
    check(lib().nexus_seal_ciphertext_save(w.ctypes.data_as(u64), size, limbs, log_n, float(scale),
                                           pid.ctypes.data_as(u64), int(is_ntt_form), None, 0, C.byref(nbytes)),
          "nexus_seal_ciphertext_save")
    out = np.zeros(nbytes.value, dtype=np.uint8)
    check(lib().nexus_seal_ciphertext_save(w.ctypes.data_as(u64), size, limbs, log_n, float(scale),
                                           pid.ctypes.data_as(u64), int(is_ntt_form), out.ctypes.data,
                                           out.size, C.byref(nbytes)), "nexus_seal_ciphertext_save")
    return out.tobytes()


def seal_load(data: bytes):
    """Ciphertext::load: (words [size][limbs][N], scale, parms_id, is_ntt_form)."""
    buf = np.frombuffer(data, dtype=np.uint8)
    size, limbs, log_n, ntt = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    scale = C.c_double()
    pid = np.zeros(4, dtype=np.uint64)
    u64 = C.POINTER(C.c_uint64)
    args = (C.byref(size), C.byref(limbs), C.byref(log_n), C.byref(scale), pid.ctypes.data_as(u64), C.byref(ntt))
    check(lib().nexus_seal_ciphertext_load(buf.ctypes.data, buf.size, None, 0, *args), "nexus_seal_ciphertext_load")
    words = np.zeros((size.value, limbs.value, 1 << log_n.value), dtype=np.uint64)
    check(lib().nexus_seal_ciphertext_load(buf.ctypes.data, buf.size, words.ctypes.data, words.size, *args),
          "nexus_seal_ciphertext_load")
    return words, scale.value, pid, bool(ntt.value)


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

    def add_galois_key(self, elt: int, key) -> None:
        self._keys.append(key)
        check(lib().nexus_evaluator_add_galois_key(self._h, int(elt), key.data_ptr()),
              "nexus_evaluator_add_galois_key")

    def set_hoisting(self, enable: bool) -> None:
        """Share one decomposition between rotations of one ciphertext (default
        on; off saves the permuted key copies; the words are the same)."""
        check(lib().nexus_evaluator_set_hoisting(self._h, 1 if enable else 0), "nexus_evaluator_set_hoisting")

    def rotate_vector_many(self, x: Ciphertext, steps) -> list:
        """rotate_vector(x, s) for every s in steps (one shared decomposition
        of x where that is exact)."""
        steps = [int(v) for v in steps]
        res = [Ciphertext(self.ctx) for _ in steps]
        arr = (C.c_int * len(steps))(*steps)
        out = (C.c_void_p * len(res))(*[r.handle.value for r in res])
        check(lib().nexus_rotate_vector_many(self._h, x.handle, arr, len(steps), out), "nexus_rotate_vector_many")
        return res

    def rotate_vector_many_batch(self, cts, steps) -> list:
        """[[rotate_vector(c, s) for c in cts] for s in steps], in lockstep
        (one shared decomposition for the batch)."""
        steps = [int(v) for v in steps]
        res = [[Ciphertext(self.ctx) for _ in cts] for _ in steps]
        a = (C.c_void_p * len(cts))(*[c.handle.value for c in cts])
        arr = (C.c_int * max(1, len(steps)))(*steps)
        flat = [r for row in res for r in row]
        out = (C.c_void_p * max(1, len(flat)))(*[r.handle.value for r in flat])
        check(lib().nexus_rotate_vector_many_batch(self._h, a, len(cts), arr, len(steps), out),
              "nexus_rotate_vector_many_batch")
        return res

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

    # ---- lockstep forms: one launch per step for the whole list ------------------
    def _batch(self, fn, name, cts, *args):
        res = [Ciphertext(self.ctx) for _ in cts]
        a = (C.c_void_p * len(cts))(*[c.handle.value for c in cts])
        r = (C.c_void_p * len(res))(*[x.handle.value for x in res])
        check(fn(self._h, a, len(cts), *args, r), name)
        return res

    def gelu_batch(self, cts):
        return self._batch(lib().nexus_gelu_batch, "nexus_gelu_batch", cts)

    def softmax_batch(self, cts, length: int):
        return self._batch(lib().nexus_softmax_batch, "nexus_softmax_batch", cts, int(length))

    def layer_norm_batch(self, cts, length: int):
        return self._batch(lib().nexus_layer_norm_batch, "nexus_layer_norm_batch", cts, int(length))

    def ckks_op_batch(self, op: int, cts, a1=0, a2=0, f=0.0):
        res = [Ciphertext(self.ctx) for _ in cts]
        a = (C.c_void_p * len(cts))(*[c.handle.value for c in cts])
        r = (C.c_void_p * len(res))(*[x.handle.value for x in res])
        check(lib().nexus_ckks_op_batch(self._h, int(op), a, len(cts), int(a1), int(a2), float(f), r),
              "nexus_ckks_op_batch")
        return res

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


BOOT_MODRAISE, BOOT_COEFFTOSLOT, BOOT_MODULAR_REDUCTION, BOOT_SLOTTOCOEFF, BOOT_SET_INITIAL_SCALE = range(5)


class Bootstrapper:
    """Bootstrapper (src/bootstrapping/Bootstrapper.h:52-69) over an Evaluator
    whose keys include the relinearisation key and the Galois keys of
    ``rotation_steps()``."""

    def __init__(self, evaluator: Evaluator, loge: int, logn: int, logNh: int, L: int, final_scale: float,
                 boundary_K: int, sin_cos_deg: int, scale_factor: int, inverse_deg: int):
        self.ev = evaluator
        self.ctx = evaluator.ctx
        self.params = dict(boundary_k=boundary_K, deg=sin_cos_deg, loge=loge, double_angle=scale_factor,
                           inverse_deg=inverse_deg)
        h = C.c_void_p()
        check(lib().nexus_bootstrapper_create(evaluator._h, loge, logn, logNh, L, float(final_scale), boundary_K,
                                              sin_cos_deg, scale_factor, inverse_deg, C.byref(h)),
              "nexus_bootstrapper_create")
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nexus_bootstrapper_destroy(self._h)
            self._h = None

    def prepare_mod_polynomial(self, table: dict | None = None):
        """Load the EvalMod heap (nexus_gb300.remez.load_table for this
        Bootstrapper's parameters unless a table is given), and for
        inverse_deg > 1 the inverse-sine polynomial."""
        from .remez import load_table
        t = table or load_table(**self.params)
        size = (1 << (t["heap_m"] + 1)) - 1
        lens = (C.c_int * size)(*[len(t["nodes"].get(i, [])) for i in range(size)])
        flat = [c for i in range(size) for c in t["nodes"].get(i, [])]
        coeffs = (C.c_double * len(flat))(*flat)
        check(lib().nexus_bootstrapper_prepare_mod_polynomial(self._h, t["heap_k"], t["heap_m"], lens, coeffs,
                                                              float(t["scale_inverse_coeff"])),
              "nexus_bootstrapper_prepare_mod_polynomial")
        inv = t.get("inverse")
        if inv is not None:
            d = int(inv["deg"])
            power = (C.c_double * (d + 1))(*inv["power"])
            if d > 3:
                isize = (1 << (inv["heap_m"] + 1)) - 1
                ilens = (C.c_int * isize)(*[len(inv["nodes"].get(i, [])) for i in range(isize)])
                iflat = [c for i in range(isize) for c in inv["nodes"].get(i, [])]
                icoeffs = (C.c_double * len(iflat))(*iflat)
                hk, hm = inv["heap_k"], inv["heap_m"]
            else:
                ilens, icoeffs, hk, hm = None, None, 0, 0
            check(lib().nexus_bootstrapper_set_inverse_polynomial(self._h, d, power, hk, hm, ilens, icoeffs),
                  "nexus_bootstrapper_set_inverse_polynomial")

    def addLeftRotKeys_Linear_to_vector_3(self, gal_steps_vector: list) -> None:
        cap = len(gal_steps_vector) + 256
        arr = (C.c_int * cap)(*gal_steps_vector)
        cnt = C.c_int(len(gal_steps_vector))
        check(lib().nexus_bootstrapper_add_rot_steps(self._h, arr, C.byref(cnt), cap),
              "nexus_bootstrapper_add_rot_steps")
        gal_steps_vector[:] = list(arr[:cnt.value])

    def rotation_steps(self, log_nh: int) -> list:
        """The reference driver's key steps (src/bootstrapping.cpp:111-118):
        0, 2^i for i < logNh, then addLeftRotKeys_Linear_to_vector_3."""
        steps = [0] + [1 << i for i in range(log_nh)]
        self.addLeftRotKeys_Linear_to_vector_3(steps)
        return steps

    def generate_LT_coefficient_3(self):
        check(lib().nexus_bootstrapper_generate_lt(self._h), "nexus_bootstrapper_generate_lt")

    def bootstrap_3(self, ct: Ciphertext) -> Ciphertext:
        """Refresh ``ct`` (one data limb; modulus-raised in place as in the
        reference) and return the new ciphertext."""
        rtn = Ciphertext(self.ctx)
        check(lib().nexus_bootstrap(self._h, ct.handle, rtn.handle), "nexus_bootstrap")
        return rtn

    def bootstrap_batch(self, cts: list, out: list | None = None) -> list:
        """bootstrap_3 of every ciphertext, run in lockstep (one launch per
        operation for the whole batch, each key read once); the inputs are
        left unchanged.  ``out``: ciphertexts to write (kept buffers when
        already of the result's size), else new ones."""
        res = out if out is not None else [Ciphertext(self.ctx) for _ in cts]
        if len(res) != len(cts):
            raise ValueError("one output per input")
        a = (C.c_void_p * len(cts))(*[c.handle.value for c in cts])
        r = (C.c_void_p * len(res))(*[x.handle.value for x in res])
        check(lib().nexus_bootstrap_batch(self._h, a, len(cts), r), "nexus_bootstrap_batch")
        return res

    def bootstrap_real_batch(self, cts: list, out: list | None = None) -> list:
        """Refresh ciphertexts of real slot values two per bootstrap
        (nexus_bootstrap_real_batch): pairs share one bootstrap_3 of
        c0 + X^(N/2) c1 and are split by a conjugation."""
        res = out if out is not None else [Ciphertext(self.ctx) for _ in cts]
        if len(res) != len(cts):
            raise ValueError("one output per input")
        a = (C.c_void_p * len(cts))(*[c.handle.value for c in cts])
        r = (C.c_void_p * len(res))(*[x.handle.value for x in res])
        check(lib().nexus_bootstrap_real_batch(self._h, a, len(cts), r), "nexus_bootstrap_real_batch")
        return res

    def argmax(self, x: Ciphertext, length: int) -> Ciphertext:
        """ArgmaxEvaluator::argmax (src/argmax.cpp) over slots 0..length-1 of x
        (x is updated in place as in the reference)."""
        res = Ciphertext(self.ctx)
        check(lib().nexus_argmax(self._h, x.handle, int(length), res.handle), "nexus_argmax")
        return res

    def argmax_batch(self, xs: list, length: int) -> list:
        """argmax of every ciphertext in lockstep (each x updated in place as
        the single form does)."""
        res = [Ciphertext(self.ctx) for _ in xs]
        a = (C.c_void_p * len(xs))(*[c.handle.value for c in xs])
        r = (C.c_void_p * len(res))(*[c.handle.value for c in res])
        check(lib().nexus_argmax_batch(self._h, a, len(xs), int(length), r), "nexus_argmax_batch")
        return res

    def stage(self, stage: int, a: Ciphertext, b: Ciphertext | None = None):
        r1, r2 = Ciphertext(self.ctx), Ciphertext(self.ctx)
        check(lib().nexus_bootstrapper_stage(self._h, stage, a.handle, None if b is None else b.handle, r1.handle,
                                             r2.handle), "nexus_bootstrapper_stage")
        return r1, r2

    def stage_batch(self, stage: int, a: list, b: list | None = None):
        """``stage`` run in lockstep over the ciphertexts ``a`` (and ``b``);
        returns the lists (r1, r2)."""
        cnt = len(a)
        r1 = [Ciphertext(self.ctx) for _ in a]
        r2 = [Ciphertext(self.ctx) for _ in a]

        def arr(xs):
            return (C.c_void_p * cnt)(*[x.handle.value for x in xs])
        check(lib().nexus_bootstrapper_stage_batch(self._h, stage, arr(a), None if b is None else arr(b), cnt,
                                                   arr(r1), arr(r2)), "nexus_bootstrapper_stage_batch")
        return r1, r2

    def cached_plaintexts(self) -> int:
        n = C.c_uint64()
        check(lib().nexus_bootstrapper_cached_plaintexts(self._h, C.byref(n)), "nexus_bootstrapper_cached_plaintexts")
        return n.value


def lt_coefficients_3(logn: int, log_nh: int, boundary_k: int, which: int) -> np.ndarray:
    """The engine's host-computed LT diagonals (complex [count][len])."""
    cnt, ln = C.c_int(), C.c_int()
    check(lib().nexus_lt_coefficients_3(logn, log_nh, boundary_k, which, None, C.byref(cnt), C.byref(ln)),
          "nexus_lt_coefficients_3")
    out = np.zeros((cnt.value, ln.value, 2))
    check(lib().nexus_lt_coefficients_3(logn, log_nh, boundary_k, which, out.ctypes.data, C.byref(cnt),
                                        C.byref(ln)), "nexus_lt_coefficients_3")
    return out


class Graph:
    """CUDA graph of the engine calls made on ``stream`` inside the ``with``
    block (nexus_graph_capture_begin / _end); ``launch()`` replays their
    device work on the same ciphertext handles.  Run the calls once before
    capturing, so that caches and grown buffers already exist.  Between
    launches only reload the captured handles (same size and level); a
    direct call that gives one of them a new buffer leaves the graph pointing
    at freed memory, so direct calls use handles of their own."""

    def __init__(self, stream):
        if stream is None:
            raise ValueError("capture needs the evaluator's own stream, not the legacy default stream")
        self.stream = stream
        self._h = None

    def __enter__(self):
        check(lib().nexus_graph_capture_begin(_stream_ptr(self.stream)), "nexus_graph_capture_begin")
        return self

    def __exit__(self, exc_type, exc, tb):
        h = C.c_void_p()
        rc = lib().nexus_graph_capture_end(_stream_ptr(self.stream), C.byref(h))
        if exc_type is not None:
            if rc == 0:
                lib().nexus_graph_destroy(h)
            return False
        check(rc, "nexus_graph_capture_end")
        self._h = h
        return False

    def launch(self, stream=None) -> None:
        check(lib().nexus_graph_launch(self._h, _stream_ptr(self.stream if stream is None else stream)),
              "nexus_graph_launch")

    def info(self) -> dict:
        nodes, kernels, allocs = C.c_size_t(), C.c_size_t(), C.c_size_t()
        check(lib().nexus_graph_info(self._h, C.byref(nodes), C.byref(kernels), C.byref(allocs)), "nexus_graph_info")
        return {"nodes": nodes.value, "kernel_nodes": kernels.value, "alloc_nodes": allocs.value}

    def __del__(self):
        if getattr(self, "_h", None):
            lib().nexus_graph_destroy(self._h)
            self._h = None
