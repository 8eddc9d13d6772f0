"""Micro-benchmarks of the engine's hot path on synthetic data (one GPU).

    python -m nexus_gb300.probe keyswitch [--batch B] [--limbs L] [--reps R] [--once]
    python -m nexus_gb300.probe stages [--batch B] [--reps R]

keyswitch: nexus_switch_key_batch at N=2^16 on the bootstrap prime chain
(51 + 16x46 + 14x51 bits + a 51-bit special prime), B ciphertexts at L limbs
under one random key; prints milliseconds per call and per ciphertext.

stages: the full-slot bootstrap at N=2^16 split into its stages (modulus
raise, CoeffToSlot, EvalMod on both halves, SlotToCoeff), single-ciphertext
and lockstep over B ciphertexts; prints milliseconds per bootstrap.

Both print, on stderr, the engine's launch counter around the measured part
(``skip=`` launches before it, then the launches of each part), so a kernel
profiler can select exactly those launches.  Inputs and keys are seeded
synthetic values; nothing here is a correctness check.
"""
from __future__ import annotations

import argparse
import sys
import time

BOOT_LOGN = 16
BOOT_BITS = [51] + [46] * 16 + [51] * 14 + [51]
BOOT_SCALE = 2.0 ** 46
BOOT_PARAMS = dict(loge=10, logn=BOOT_LOGN - 1, logNh=BOOT_LOGN - 1, L=len(BOOT_BITS) - 2, final_scale=BOOT_SCALE,
                   boundary_K=25, sin_cos_deg=59, scale_factor=2, inverse_deg=1)


def _timed(f, sync):
    sync()
    t0 = time.perf_counter()
    r = f()
    sync()
    return r, (time.perf_counter() - t0) * 1e3


def keyswitch(batch: int, limbs: int, reps: int, once: bool) -> None:
    import torch

    import nexus_gb300 as ng
    n = 1 << BOOT_LOGN
    qs = ng.create_coeff_modulus(n, BOOT_BITS)
    if not 1 <= limbs <= len(qs) - 1:
        raise SystemExit(f"--limbs must be in [1, {len(qs) - 1}]")
    ctx = ng.Context(BOOT_LOGN, qs)
    k = len(qs)
    g = torch.Generator(device="cuda").manual_seed(1)
    qd = torch.tensor(qs, dtype=torch.int64, device="cuda")

    def rnd(lead, rows, primes):
        x = torch.randint(0, 2 ** 62, tuple(lead) + (rows, n), device="cuda", dtype=torch.int64, generator=g)
        return x % primes.view(rows, 1)

    key = rnd((k - 1, 2), k, qd)
    cts, tg = rnd((batch, 2), limbs, qd[:limbs]), rnd((batch,), limbs, qd[:limbs])
    if not once:
        for _ in range(2):
            ctx.switch_key_batch(cts, tg, key)
    torch.cuda.synchronize()
    a = ng.kernel_launches()
    _, ms = _timed(lambda: [ctx.switch_key_batch(cts, tg, key) for _ in range(1 if once else reps)],
                   torch.cuda.synchronize)
    print(f"skip={a} keyswitch={ng.kernel_launches() - a}", file=sys.stderr)
    calls = 1 if once else reps
    print(f"keyswitch N=2^16 limbs={limbs} batch={batch}: {ms / calls:.3f} ms per call, "
          f"{ms / calls / batch:.3f} ms per ciphertext")


def stages(batch: int, reps: int) -> None:
    import numpy as np
    import torch

    import nexus_gb300 as ng
    from nexus_gb300.operators import (BOOT_COEFFTOSLOT, BOOT_MODRAISE, BOOT_MODULAR_REDUCTION,
                                       BOOT_SET_INITIAL_SCALE, BOOT_SLOTTOCOEFF, Bootstrapper, Ciphertext, Evaluator)
    n = 1 << BOOT_LOGN
    qs = ng.create_coeff_modulus(n, BOOT_BITS)
    ctx = ng.Context(BOOT_LOGN, qs)
    sk = ctx.keygen_secret(seed=71, hamming_weight=192)
    ev = Evaluator(ctx, BOOT_SCALE, ctx.keygen_relin(sk, seed=72))
    bs = Bootstrapper(ev, **BOOT_PARAMS)
    for i, st in enumerate(bs.rotation_steps(BOOT_LOGN - 1)):
        e = ctx.galois_elt(st)
        ev.add_galois_key(e, ctx.keygen_galois(sk, e, seed=1000 + i))
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    top = len(qs) - 1
    rng = np.random.default_rng(1)
    pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
    ins = []
    for i in range(batch):
        ctx.encode(rng.uniform(-1, 1, n // 2), BOOT_SCALE, top, pt)
        ins.append(ctx.encrypt_symmetric(sk, pt, top, 600 + i)[:, :1, :].contiguous())
    sync = torch.cuda.synchronize
    q0 = float(qs[0])

    def single(x0):
        x = Ciphertext.from_device(ctx, x0.clone(), BOOT_SCALE)
        bs.stage(BOOT_SET_INITIAL_SCALE, x)
        t = {}
        _, t["modraise"] = _timed(lambda: bs.stage(BOOT_MODRAISE, x), sync)
        x = Ciphertext.from_device(ctx, x.to_device(), q0)
        (r1, r2), t["coefftoslot"] = _timed(lambda: bs.stage(BOOT_COEFFTOSLOT, x), sync)
        (m1, _), t["evalmod_1"] = _timed(lambda: bs.stage(BOOT_MODULAR_REDUCTION, r1), sync)
        (m2, _), t["evalmod_2"] = _timed(lambda: bs.stage(BOOT_MODULAR_REDUCTION, r2), sync)
        _, t["slottocoeff"] = _timed(lambda: bs.stage(BOOT_SLOTTOCOEFF, m1, m2), sync)
        return t

    def lockstep():
        xs = [Ciphertext.from_device(ctx, x.clone(), BOOT_SCALE) for x in ins]
        bs.stage_batch(BOOT_SET_INITIAL_SCALE, xs)
        t, c = {}, {}
        _, t["modraise"] = _timed(lambda: bs.stage_batch(BOOT_MODRAISE, xs), sync)
        xs = [Ciphertext.from_device(ctx, x.to_device(), q0) for x in xs]
        skip = ng.kernel_launches()
        (r1, r2), t["coefftoslot"] = _timed(lambda: bs.stage_batch(BOOT_COEFFTOSLOT, xs), sync)
        c["coefftoslot"] = ng.kernel_launches() - skip
        b = ng.kernel_launches()
        (m1, _), t["evalmod_1"] = _timed(lambda: bs.stage_batch(BOOT_MODULAR_REDUCTION, r1), sync)
        c["evalmod_1"] = ng.kernel_launches() - b
        b = ng.kernel_launches()
        (m2, _), t["evalmod_2"] = _timed(lambda: bs.stage_batch(BOOT_MODULAR_REDUCTION, r2), sync)
        c["evalmod_2"] = ng.kernel_launches() - b
        b = ng.kernel_launches()
        _, t["slottocoeff"] = _timed(lambda: bs.stage_batch(BOOT_SLOTTOCOEFF, m1, m2), sync)
        c["slottocoeff"] = ng.kernel_launches() - b
        return t, c, skip

    single(ins[0])          # first use builds the plaintext and hoisting caches
    lockstep()
    for r in range(reps):
        t = single(ins[0])
        print("single:   " + ", ".join(f"{k} {v:.2f}" for k, v in t.items()) +
              f"; total {sum(t.values()):.2f} ms per bootstrap", flush=True)
    for r in range(reps):
        t, c, skip = lockstep()
        print(f"lockstep x{batch}: " + ", ".join(f"{k} {v / batch:.2f}" for k, v in t.items()) +
              f"; total {sum(t.values()) / batch:.2f} ms per bootstrap", flush=True)
        if r == reps - 1:
            print(f"skip={skip} " + " ".join(f"{k}={v}" for k, v in c.items()), file=sys.stderr)


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(prog="python -m nexus_gb300.probe", description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    k = sub.add_parser("keyswitch")
    k.add_argument("--batch", type=int, default=4)
    k.add_argument("--limbs", type=int, default=31)
    k.add_argument("--reps", type=int, default=5)
    k.add_argument("--once", action="store_true", help="one call, no warm-up (for a kernel profiler)")
    s = sub.add_parser("stages")
    s.add_argument("--batch", type=int, default=16)
    s.add_argument("--reps", type=int, default=2)
    args = ap.parse_args(argv)
    if args.cmd == "keyswitch":
        keyswitch(args.batch, args.limbs, args.reps, args.once)
    else:
        stages(args.batch, args.reps)


if __name__ == "__main__":
    main()
