"""EvalMod polynomial table for bootstrapping: minimax cosine + its BSGS heap.

Restates the setup NEXUS runs once per Bootstrapper in high precision
(NTL RR in the reference, mpmath here):

* ``RemezCos`` (src/bootstrapping/RemezCos.h:12-17): minimax polynomial of
  degree ``deg`` in the Chebyshev basis of x/K approximating
  cos(2*pi*(x - 1/4) / 2^r) on the union of [i - 2^-loge, i + 2^-loge],
  |i| < K, where r is the number of double-angle steps.  The exchange
  follows common/Remez.cpp: initial reference from ``better_initialize``
  (:21-127), levelled solve (``getcoeffwitherr`` :175-213), local extrema on
  every interval, the alternating-maximum selection of ``choosemaxs``
  (:434-560), stop when (max_err - min_err)/min_err <= 2^-``log_approx``.
  The extrema are located by golden-section search to full working
  precision (the reference scans with a step of width/2^9.5 and refines with
  10 bisections), so the result is the minimax polynomial itself.
* ``RemezArcsin`` (RemezArcsin.h:5-13) of degree ``inverse_deg`` on
  [-w, w] with w = sin(2*pi*2^-loge).  For degree 1 its linear coefficient
  becomes ``scale_inverse_coeff`` after ``r`` square roots and scales the
  cosine polynomial (ModularReducer.cpp:11-16,38-46); for higher degrees the
  cosine stays unscaled and the inverse-sine polynomial is evaluated after
  the double angles (:62-73), directly from its power-basis coefficients up
  to degree 3 and through an odd heap (``generate_poly_heap_odd``,
  common/Polynomial.cpp:207-210, ``oddbabycount`` common/func.cpp:95-118)
  above.
* ``Polynomial::generate_poly_heap`` (common/Polynomial.cpp:168-214,
  ``babycount`` common/func.cpp:120-142): the polynomial is split by
  T_{k 2^(m-1)}, ..., T_k into a heap whose leaves (degree < k) are what
  ``homomorphic_poly_evaluation`` (:255-485) encodes, as doubles.

The table is data: ``load_table`` reads the committed JSON and needs no
mpmath; ``python -m nexus_gb300.remez`` regenerates it (mpmath required).
"""
from __future__ import annotations

import json
import math
from pathlib import Path

DATA_DIR = Path(__file__).resolve().parent / "data"


def table_name(boundary_k: int, deg: int, loge: int, double_angle: int, inverse_deg: int) -> str:
    return f"evalmod_K{boundary_k}_deg{deg}_loge{loge}_da{double_angle}_inv{inverse_deg}.json"


def babycount(deg: int) -> tuple[int, int]:
    """(k, m) of common/func.cpp:120-142: baby steps T_1..T_{k-1}, m giant steps."""
    mink = 2
    d_over_k = deg / mink
    min_mul = math.ceil(math.log2(d_over_k)) + mink + math.ceil(d_over_k) - 3
    minm = math.ceil(math.log2(d_over_k))
    i = 3
    while i < 2 * math.sqrt(deg):
        d_over_k = deg / i
        lg = math.ceil(math.log2(d_over_k))
        cur = lg + i + math.ceil(d_over_k) - 3
        if min_mul > cur:
            mink, min_mul, minm = i, cur, lg
        i += 1
    return mink, minm


def oddbabycount(deg: int) -> tuple[int, int]:
    """(k, m) of common/func.cpp:95-118 for an odd polynomial's heap: even k,
    the split whose depth matches ceil(log2(deg)) with the fewest estimated
    products (natural log in its ceil(log(k)) term, as written there)."""
    mink = minm = 0
    mind = 0
    mineval = 100000
    for k in range(2, deg + 1, 2):
        m = 1
        while (1 << m) * k < deg:
            m += 1
        if math.ceil(math.log(k) / math.log(2)) + m != math.ceil(math.log(deg) / math.log(2)):
            continue
        ev = (math.ceil(deg / k) + k // 2 - 5 + m + math.ceil(math.log(k))
              + max(3.0 - m, math.ceil(deg / (1.5 * (1 << (m - 1)) * k))))
        depth = math.ceil(math.log(k) / math.log(2)) + m
        if mineval > ev:
            mineval, mink, minm, mind = int(ev), k, m, depth
        elif mineval == ev and mind > depth:
            mink, minm, mind = k, m, depth
    return mink, minm


def _parse_heap(nodes: dict) -> dict:
    return {int(k): [float.fromhex(c) for c in v] for k, v in nodes.items()}


def load_table(boundary_k=25, deg=59, loge=10, double_angle=2, inverse_deg=1) -> dict:
    """The committed heap table: {"heap_k", "heap_m", "nodes": {index: [cheb coeffs]},
    "scale_inverse_coeff", ...} with every coefficient the double the
    homomorphic evaluation encodes.  With inverse_deg > 1 it also holds
    "inverse": {"deg", "power": [power-basis coefficients], and for deg > 3
    "heap_k", "heap_m", "nodes"} -- the inverse-sine polynomial evaluated
    after the double angles."""
    path = DATA_DIR / table_name(boundary_k, deg, loge, double_angle, inverse_deg)
    if not path.exists():
        raise FileNotFoundError(f"no EvalMod table for K={boundary_k} deg={deg} loge={loge} "
                                f"double_angle={double_angle} inverse_deg={inverse_deg}; "
                                "generate it with python -m nexus_gb300.remez")
    with open(path) as f:
        t = json.load(f)
    t["nodes"] = _parse_heap(t["nodes"])
    t["scale_inverse_coeff"] = float.fromhex(t["scale_inverse_coeff"])
    inv = t.get("inverse")
    if inv is not None:
        inv["power"] = [float.fromhex(c) for c in inv["power"]]
        if "nodes" in inv:
            inv["nodes"] = _parse_heap(inv["nodes"])
    return t


# --------------------------------------------------------------------------
# generation (mpmath)
# --------------------------------------------------------------------------

def _better_initialize(boundary_k: int, log_width: float, deg: int):
    """Initial reference of Remez::better_initialize (Remez.cpp:21-127): a
    per-interval node count from an error-bound heuristic, then Chebyshev
    nodes inside each interval."""
    import mpmath as mp

    k = boundary_k
    nodecount = [1] * k
    deg_bdd = deg + 2
    tot_deg = 2 * k - 1
    err = 2.0 ** (-log_width)
    temp = -sum(math.log2(i) for i in range(1, 2 * k)) + (2 * k - 1) * math.log2(2 * math.pi) + math.log2(err)
    bdd = []
    for i in range(k):
        b = temp
        for j in range(1, k - i):
            b += math.log2(j + err)
        for j in range(1, k + i):
            b += math.log2(j + err)
        bdd.append(b)
    for _ in range(200):
        if tot_deg >= deg_bdd:
            break
        maxi = max(range(k), key=lambda i: (bdd[i], -i))
        if maxi != 0:
            if tot_deg + 2 > deg_bdd:
                break
            for i in range(k):
                bdd[i] -= math.log2(tot_deg + 1) + math.log2(tot_deg + 2)
                bdd[i] += 2.0 * math.log2(2.0 * math.pi)
                if i != maxi:
                    bdd[i] += math.log2(abs(i - maxi) + err) + math.log2(i + maxi + err)
                else:
                    bdd[i] += math.log2(err) - 1.0 + math.log2(2.0 * i + err)
            tot_deg += 2
        else:
            bdd[0] += -math.log2(tot_deg + 1) + math.log2(err) - 1.0 + math.log2(2.0 * math.pi)
            for i in range(1, k):
                bdd[i] += -math.log2(tot_deg + 1) + math.log2(2.0 * math.pi) + math.log2(i + err)
            tot_deg += 1
        nodecount[maxi] += 1
    if tot_deg == deg_bdd - 1:
        nodecount[0] += 1
    w = mp.mpf(2) ** (-mp.mpf(log_width))
    pts = []
    if nodecount[0] % 2:
        pts.append(mp.mpf(0))
    for i in range(k - 1, 0, -1):
        for j in range(1, nodecount[i] + 1):
            c = mp.cos((2 * j - 1) * mp.pi / (2 * nodecount[i]))
            pts += [i + w * c, -i - w * c]
    for j in range(1, nodecount[0] // 2 + 1):
        c = mp.cos((2 * j - 1) * mp.pi / (2 * nodecount[0]))
        pts += [w * c, -w * c]
    pts.sort()
    if len(pts) != deg + 2:
        raise RuntimeError(f"initial reference has {len(pts)} points, expected {deg + 2}")
    return pts


def _cheb(coeff, t):
    """sum_j coeff[j] T_j(t) (Clenshaw)."""
    b1 = b2 = 0
    for c in reversed(coeff[1:]):
        b1, b2 = 2 * t * b1 - b2 + c, b1
    return t * b1 - b2 + coeff[0]


def remez(func, boundary_k: int, width, deg: int, log_approx: int = 100, samples: int = 48,
          golden_iters: int = 90, max_iter: int = 60, log_width: float | None = None):
    """Multi-interval Remez exchange; returns (Chebyshev coefficients in x/K, levelled error)."""
    import mpmath as mp

    k = boundary_k
    intervals = [(i - width, i + width) for i in range(-(k - 1), k)]
    ref = _better_initialize(k, log_width, deg)
    tol = mp.mpf(2) ** (-log_approx)
    gr = (mp.sqrt(5) - 1) / 2
    for it in range(max_iter):
        # levelled solve: sum_j c_j T_j(x_i/K) + (-1)^i E = f(x_i)
        n = deg + 2
        m = mp.matrix(n, n)
        rhs = mp.matrix(n, 1)
        for i, x in enumerate(ref):
            t = x / k
            tp, tc = mp.mpf(1), t
            m[i, 0] = 1
            if deg >= 1:
                m[i, 1] = t
            for j in range(2, deg + 1):
                tp, tc = tc, 2 * t * tc - tp
                m[i, j] = tc
            m[i, deg + 1] = 1 if i % 2 == 0 else -1
            rhs[i] = func(x)
        sol = mp.lu_solve(m, rhs)
        coeff = [sol[j] for j in range(deg + 1)]

        def err(x):
            return _cheb(coeff, x / k) - func(x)

        # local extrema of the error on every interval
        ext = []
        for a, b in intervals:
            xs = [a + (b - a) * s / (samples - 1) for s in range(samples)]
            ys = [err(x) for x in xs]
            for s in range(samples):
                y = ys[s]
                sg = 1 if y > 0 else -1
                left = ys[s - 1] * sg if s > 0 else None
                right = ys[s + 1] * sg if s < samples - 1 else None
                if (left is not None and left > y * sg) or (right is not None and right > y * sg):
                    continue
                if s == 0 or s == samples - 1:
                    ext.append((xs[s], y))
                    continue
                lo, hi = xs[s - 1], xs[s + 1]
                c = hi - gr * (hi - lo)
                d = lo + gr * (hi - lo)
                fc, fd = err(c) * sg, err(d) * sg
                for _ in range(golden_iters):
                    if fc > fd:
                        hi, d, fd = d, c, fc
                        c = hi - gr * (hi - lo)
                        fc = err(c) * sg
                    else:
                        lo, c, fc = c, d, fd
                        d = lo + gr * (hi - lo)
                        fd = err(d) * sg
                xm = (lo + hi) / 2
                ext.append((xm, err(xm)))
        ext.sort(key=lambda p: p[0])
        # keep the largest of every run of equal sign
        alt = []
        for x, y in ext:
            if alt and (alt[-1][1] > 0) == (y > 0):
                if abs(y) > abs(alt[-1][1]):
                    alt[-1] = (x, y)
            else:
                alt.append((x, y))
        max_err = max(abs(y) for _, y in ext)
        # choosemaxs: trim to deg + 2 alternating points
        while len(alt) > deg + 2:
            if len(alt) == deg + 3:
                alt = alt[:-1] if abs(alt[0][1]) > abs(alt[-1][1]) else alt[1:]
            else:
                sums = [abs(alt[i][1]) + abs(alt[i + 1][1]) for i in range(len(alt) - 1)]
                mi = min(range(len(sums)), key=lambda i: sums[i])
                if mi == 0:
                    alt = alt[1:]
                elif mi == len(alt) - 2:
                    alt = alt[:-1]
                else:
                    alt = alt[:mi] + alt[mi + 2:]
        if len(alt) < deg + 2:
            raise RuntimeError(f"Remez: only {len(alt)} alternating extrema at iteration {it}")
        min_err = min(abs(y) for _, y in alt)
        ref = [x for x, _ in alt]
        if (max_err - min_err) / min_err <= tol:
            return coeff, max_err, it + 1
    raise RuntimeError("Remez did not converge")


class _Poly:
    """Power-basis polynomial with its Chebyshev coefficients (common/Polynomial.h)."""

    def __init__(self, coeff):
        self.coeff = list(coeff)
        self.cheb = None

    @property
    def deg(self):
        return len(self.coeff) - 1


def _chebyshev_power(deg: int):
    """Power-basis coefficients of T_deg (common/Polynomial.cpp:910-937)."""
    import mpmath as mp

    t0, t1 = [mp.mpf(1)], [mp.mpf(0), mp.mpf(1)]
    if deg == 0:
        return t0
    for _ in range(2, deg + 1):
        t2 = [mp.mpf(0)] + [2 * c for c in t1]
        for i, c in enumerate(t0):
            t2[i] -= c
        t0, t1 = t1, t2
    return t1


def _cheb_to_power(cheb):
    import mpmath as mp

    out = [mp.mpf(0)] * len(cheb)
    for i, c in enumerate(cheb):
        for j, t in enumerate(_chebyshev_power(i)):
            out[j] += t * c
    return out


def _power_to_cheb(coeff):
    """Polynomial::power_to_cheb (:93-107): peel T_i from the top degree down."""
    tmp = list(coeff)
    deg = len(coeff) - 1
    cheb = [None] * (deg + 1)
    for i in range(deg, -1, -1):
        t = _chebyshev_power(i)
        cheb[i] = tmp[i] / t[i]
        for j in range(i + 1):
            tmp[j] -= t[j] * cheb[i]
    return cheb


def _divide(target: _Poly, divider_deg: int):
    """divide_poly (:883-908) by T_divider_deg: quotient and remainder in the power basis."""
    import mpmath as mp

    div = _chebyshev_power(divider_deg)
    if target.deg < divider_deg:
        return _Poly([mp.mpf(0)]), _Poly(target.coeff)
    qdeg = target.deg - divider_deg
    tmp = list(target.coeff)
    q = [mp.mpf(0)] * (qdeg + 1)
    cur = target.deg
    for i in range(qdeg, -1, -1):
        c = tmp[cur] / div[divider_deg]
        q[i] = c
        tmp[cur] = mp.mpf(0)
        for j in range(divider_deg):
            tmp[j + i] -= div[j] * c
        cur -= 1
    return _Poly(q), _Poly(tmp[:divider_deg])


def poly_heap(cheb_coeff, heap_k: int, heap_m: int) -> dict:
    """generate_poly_heap_manual (:168-205): {heap index: Chebyshev coefficients}."""
    root = _Poly(_cheb_to_power(cheb_coeff))
    root.cheb = list(cheb_coeff)
    heap = {0: root}
    chebdeg = heap_k << heap_m
    for i in range(heap_m):
        chebdeg >>= 1
        for j in range((1 << i) - 1, (1 << (i + 1)) - 1):
            node = heap.get(j)
            if node is None:
                continue
            if node.deg < chebdeg:
                heap[2 * (j + 1)] = node
            else:
                q, r = _divide(node, chebdeg)
                q.cheb = _power_to_cheb(q.coeff)
                r.cheb = _power_to_cheb(r.coeff)
                heap[2 * (j + 1) - 1] = q
                heap[2 * (j + 1)] = r
    return heap


def generate(boundary_k=25, deg=59, loge=10, double_angle=2, inverse_deg=1, prec=1000, remez_prec=320):
    """Run the setup and return the table dict (doubles as hex strings)."""
    import mpmath as mp

    if inverse_deg < 1:
        raise ValueError("inverse_deg must be at least 1")
    scale_factor = 1 << double_angle
    mp.mp.prec = remez_prec
    width = mp.mpf(2) ** (-loge)
    if scale_factor % 2 == 0:
        def fcos(x):
            return mp.cos(2 * mp.pi * (x - mp.mpf(0.25)) / scale_factor)
    else:
        def fcos(x):
            return mp.sin(2 * mp.pi * x / scale_factor)
    cheb, cos_err, cos_iters = remez(fcos, boundary_k, width, deg, log_width=float(loge))

    # RemezArcsin: degree 1 on [-w, w], w = 2^-inverse_log_width computed in doubles
    inverse_log_width = -math.log2(math.sin(2 * math.pi * math.pow(2.0, -loge)))
    w_inv = mp.mpf(math.pow(2.0, -inverse_log_width))

    def fasin(x):
        return mp.asin(x) / (2 * mp.pi)

    inv_cheb, inv_err, inv_iters = remez(fasin, 1, w_inv, inverse_deg, log_width=inverse_log_width)

    def hexheap(heap):
        return {str(idx): [float(c).hex() for c in node.cheb] for idx, node in sorted(heap.items())}

    mp.mp.prec = prec
    heap_k, heap_m = babycount(deg)
    out = {
        "boundary_K": boundary_k, "deg": deg, "loge": loge, "double_angle": double_angle,
        "inverse_deg": inverse_deg, "heap_k": heap_k, "heap_m": heap_m,
        "cos_cheb": [float(c).hex() for c in cheb],
        "cos_levelled_error": float(cos_err), "cos_remez_iterations": cos_iters,
        "arcsin_c1": float(inv_cheb[1]).hex(), "arcsin_levelled_error": float(inv_err),
    }
    if inverse_deg == 1:
        # generate_inverse_sine_polynomial (ModularReducer.cpp:38-46): the
        # linear coefficient, square-rooted once per double angle, scales
        # the cosine polynomial
        s = float(inv_cheb[1])
        for _ in range(double_angle):
            s = math.sqrt(s)
        scaled = [mp.mpf(c) * mp.mpf(s) for c in cheb]
        out["scale_inverse_coeff"] = s.hex()
        out["nodes"] = hexheap(poly_heap(scaled, heap_k, heap_m))
        return out
    # inverse_deg > 1: the cosine is used as it is, and the inverse-sine
    # polynomial (power basis for the direct forms of degree <= 3, an odd
    # heap for higher degrees) follows the unscaled double angles
    out["scale_inverse_coeff"] = (1.0).hex()
    out["nodes"] = hexheap(poly_heap(cheb, heap_k, heap_m))
    inv = {"deg": inverse_deg, "power": [float(c).hex() for c in _cheb_to_power(inv_cheb)],
           "remez_iterations": inv_iters}
    if inverse_deg > 3:
        ik, im = oddbabycount(inverse_deg)
        inv["heap_k"], inv["heap_m"] = ik, im
        inv["nodes"] = hexheap(poly_heap(inv_cheb, ik, im))
    out["inverse"] = inv
    return out


def main(argv=None):
    import argparse

    ap = argparse.ArgumentParser(description="regenerate an EvalMod heap table (needs mpmath)")
    ap.add_argument("--K", type=int, default=25)
    ap.add_argument("--deg", type=int, default=59)
    ap.add_argument("--loge", type=int, default=10)
    ap.add_argument("--double-angle", type=int, default=2)
    ap.add_argument("--inverse-deg", type=int, default=1)
    a = ap.parse_args(argv)
    t = generate(a.K, a.deg, a.loge, a.double_angle, a.inverse_deg)
    DATA_DIR.mkdir(exist_ok=True)
    path = DATA_DIR / table_name(a.K, a.deg, a.loge, a.double_angle, a.inverse_deg)
    with open(path, "w") as f:
        json.dump(t, f, indent=1)
    print(f"wrote {path}: levelled error {t['cos_levelled_error']:.3e} "
          f"after {t['cos_remez_iterations']} iterations")


if __name__ == "__main__":
    main()
