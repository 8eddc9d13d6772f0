"""CUDA-graph capture of engine calls (nexus_graph_*), through the C ABI.

A lockstep bootstrap (nexus_bootstrap_batch) of two ciphertexts at N=2^13 on
the bootstrap test chain is run once, captured into a graph on the
evaluator's stream, and replayed on new inputs loaded into the captured
input handles: every replay must give exactly the words of a direct call on
the same inputs.  Output handles first sized inside the capture keep a
valid buffer across launches and after the graph is gone, and a failing call
inside a capture ends it cleanly.  GELU (single and lockstep) and the
reduced-size BERT layer are replayed the same way.
"""
import numpy as np
import pytest

from oracle import bootstrap as B
from tests.util import to_host

pytestmark = pytest.mark.gpu

LOG_N = 13
N = 1 << LOG_N
LOG_NH = LOG_N - 1
SCALE = 2.0 ** 46
BITS = [51] + [46] * 2 + [51] * 14 + [51]
PARAMS = dict(loge=10, logn=LOG_NH, logNh=LOG_NH, L=len(BITS) - 2, final_scale=SCALE, boundary_K=25,
              sin_cos_deg=59, scale_factor=2, inverse_deg=1)


@pytest.fixture(scope="module")
def env(cuda):
    import torch

    import nexus_gb300 as ng
    from nexus_gb300.operators import Bootstrapper, Evaluator
    qs = ng.create_coeff_modulus(N, BITS)
    ctx = ng.Context(LOG_N, qs)
    sk = ctx.keygen_secret(seed=51, hamming_weight=192)
    rk = ctx.keygen_relin(sk, seed=52)
    steps = B.rot_key_steps_3(LOG_NH, LOG_NH)
    gks = {ctx.galois_elt(st): ctx.keygen_galois(sk, ctx.galois_elt(st), seed=53 + i) for i, st in enumerate(steps)}
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    ev = Evaluator(ctx, SCALE, rk, gks, stream=stream)
    bs = Bootstrapper(ev, **PARAMS)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    torch.cuda.synchronize()
    return ctx, sk, ev, bs, stream


def _lowest_limb_ct(ctx, sk, seed):
    """A fresh encryption of U(-1, 1) slots reduced to its q0 limb, as a device tensor [2][1][N]."""
    import torch
    vals = np.random.default_rng(seed).uniform(-1, 1, N // 2)
    top = len(ctx.moduli) - 1
    pt = torch.empty((top, N), dtype=torch.int64, device="cuda")
    ctx.encode(vals, SCALE, top, pt)
    ct = ctx.encrypt_symmetric(sk, pt, top, seed)
    torch.cuda.synchronize()
    return ct[:, :1, :].contiguous()


def _words(cts, stream):
    stream.synchronize()
    return [c.to_numpy() for c in cts]


def test_bootstrap_batch_graph_replays_direct_words(env):
    import torch

    from nexus_gb300.operators import Ciphertext, Graph
    ctx, sk, ev, bs, stream = env
    batches = [[_lowest_limb_ct(ctx, sk, 100 + 10 * k + b) for b in range(2)] for k in range(3)]

    # direct calls on each batch
    direct = []
    for batch in batches:
        ins = [Ciphertext(ctx) for _ in batch]
        for c, t in zip(ins, batch):
            c.load(t, SCALE, stream)
        direct.append(_words(bs.bootstrap_batch(ins), stream))

    # one warm-up call sizes the outputs, then the capture
    ins = [Ciphertext(ctx) for _ in range(2)]
    outs = [Ciphertext(ctx) for _ in range(2)]
    for c, t in zip(ins, batches[0]):
        c.load(t, SCALE, stream)
    bs.bootstrap_batch(ins, outs)
    stream.synchronize()
    with Graph(stream) as g:
        bs.bootstrap_batch(ins, outs)
    info = g.info()
    assert info["kernel_nodes"] > 100
    for k in (1, 2, 0):
        for c, t in zip(ins, batches[k]):
            c.load(t, SCALE, stream)
        g.launch()
        got = _words(outs, stream)
        for a, b in zip(got, direct[k]):
            assert np.array_equal(a, b)
    torch.cuda.synchronize()


def test_outputs_first_sized_inside_the_capture(env):
    """Output handles without a buffer get a graph allocation inside the
    capture; it stays valid from launch to launch (auto-free on launch)."""
    import torch

    from nexus_gb300.operators import Ciphertext, Graph
    ctx, sk, ev, bs, stream = env
    ts = [_lowest_limb_ct(ctx, sk, 300 + k) for k in range(2)]
    ins = [Ciphertext(ctx)]
    direct = []
    for t in ts:
        ins[0].load(t, SCALE, stream)
        direct.append(_words(bs.bootstrap_batch(ins), stream)[0])   # also warms the batch-of-one caches
    fresh = [Ciphertext(ctx)]
    with Graph(stream) as g:
        bs.bootstrap_batch(ins, fresh)
    for k in (0, 1, 0):
        ins[0].load(ts[k], SCALE, stream)
        g.launch()
        assert np.array_equal(_words(fresh, stream)[0], direct[k])
    del g
    torch.cuda.synchronize()
    assert np.array_equal(_words(fresh, stream)[0], direct[0])   # the handle outlives the graph


def test_an_error_inside_the_capture_ends_it(env):
    """A call that fails inside the block (here on its arguments, before any
    device work) ends the capture and keeps no graph; the stream then runs
    direct calls as before."""
    from nexus_gb300 import NexusError
    from nexus_gb300.operators import Ciphertext, Graph
    ctx, sk, ev, bs, stream = env
    t = _lowest_limb_ct(ctx, sk, 9)
    ins = [Ciphertext(ctx)]
    ins[0].load(t, SCALE, stream)
    want = _words(bs.bootstrap_batch(ins), stream)[0]
    with pytest.raises(NexusError, match="empty"):
        with Graph(stream):
            bs.bootstrap_batch([Ciphertext(ctx)])
    assert np.array_equal(_words(bs.bootstrap_batch(ins), stream)[0], want)


@pytest.fixture(scope="module")
def gelu_env(cuda):
    import torch

    import nexus_gb300 as ng
    from nexus_gb300.operators import Evaluator
    n = 1 << 12
    qs = ng.create_coeff_modulus(n, [58] + [40] * 18 + [58])
    ctx = ng.Context(12, qs)
    sk = ctx.keygen_secret(seed=61)
    rk = ctx.keygen_relin(sk, seed=62)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    return ctx, sk, Evaluator(ctx, 2.0 ** 40, rk, stream=stream), stream


def _gelu_inputs(ctx, sk, count, seed):
    import torch
    n = ctx.n
    top = len(ctx.moduli) - 1
    out = []
    for i in range(count):
        pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
        ctx.encode(np.random.default_rng(seed + i).uniform(-5, 5, n // 2), 2.0 ** 40, top, pt)
        out.append(ctx.encrypt_symmetric(sk, pt, top, seed + i))
    torch.cuda.synchronize()
    return out


def test_gelu_graph_single_and_lockstep(gelu_env):
    """GELU's vector constants are encoded once per evaluator, so repeated
    calls wait on nothing: both forms capture, and replays on new inputs give
    the direct calls' words (single form: x is mod-switched in place, so the
    caller reloads it before each launch, as for a direct call)."""
    from nexus_gb300.operators import Ciphertext, Graph
    ctx, sk, ev, stream = gelu_env
    sets = [_gelu_inputs(ctx, sk, 2, 700 + 10 * k) for k in range(2)]

    def direct_single(t):
        x = Ciphertext(ctx)
        x.load(t, 2.0 ** 40, stream)
        return _words([ev.gelu(x)], stream)[0]

    def direct_batch(ts):
        xs = [Ciphertext(ctx) for _ in ts]
        for x, t in zip(xs, ts):
            x.load(t, 2.0 ** 40, stream)
        return _words(ev.gelu_batch(xs), stream)

    want_single = [direct_single(ts[0]) for ts in sets]      # also fills the constant cache
    want_batch = [direct_batch(ts) for ts in sets]

    x = Ciphertext(ctx)
    x.load(sets[0][0], 2.0 ** 40, stream)
    with Graph(stream) as g1:
        y = ev.gelu(x)
    xs = [Ciphertext(ctx) for _ in range(2)]
    for c, t in zip(xs, sets[0]):
        c.load(t, 2.0 ** 40, stream)
    with Graph(stream) as g2:
        ys = ev.gelu_batch(xs)
    for k in (1, 0):
        x.load(sets[k][0], 2.0 ** 40, stream)
        g1.launch()
        assert np.array_equal(_words([y], stream)[0], want_single[k])
        for c, t in zip(xs, sets[k]):
            c.load(t, 2.0 ** 40, stream)
        g2.launch()
        for a, b in zip(_words(ys, stream), want_batch[k]):
            assert np.array_equal(a, b)


def test_bert_layer_graph_matches_oracle(cuda):
    """The whole lockstep encoder layer (the reduced size of
    tests/golden/bert_digests.json: N=2^13, hidden 64, requests of 40 | 8 + 32
    tokens) captured as one graph: replays on the captured inputs give the
    oracle's output digests, the same as the direct call."""
    import torch

    import nexus_gb300 as ng
    from nexus_gb300 import bert as NB
    from nexus_gb300.operators import Bootstrapper, Ciphertext, Evaluator, Graph
    from tests.test_bert_gpu import DOC, _lane_digests, _shape, _want
    c = DOC
    n = 1 << c["log_n"]
    qs = [int(q) for q in c["moduli"]]
    ctx = ng.Context(c["log_n"], qs)
    seed = np.array(c["seed"], dtype=np.uint64)
    scale = 2.0 ** c["scale_log2"]
    sk = ctx.seal_keygen_secret(seed, c["hamming_weight"])
    rk = ctx.seal_keygen_relin(sk, seed)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream()
    ev = Evaluator(ctx, scale, rk, stream=stream)
    log_nh = c["log_n"] - 1
    bs = Bootstrapper(ev, c["loge"], log_nh, log_nh, len(qs) - 2, scale, c["boundary_K"], c["sin_cos_deg"],
                      c["scale_factor"], c["inverse_deg"])
    sh = _shape()
    w = NB.random_weights(sh, np.random.default_rng(c["weight_seed"]))
    rng = np.random.default_rng(c["token_seed"])
    tokens = [[rng.normal(0, 1, (L, sh.hidden)) for (_, L) in lane] for lane in sh.lanes]
    steps = bs.rotation_steps(log_nh)
    bs.prepare_mod_polynomial()
    bs.generate_LT_coefficient_3()
    layer = NB.BertLayer(bs, sh, w)
    for s in steps + [s for s in layer.rotation_steps() if s not in steps]:
        e = ctx.galois_elt(s)
        ev.add_galois_key(e, ctx.seal_keygen_galois(sk, e, seed))
    top = len(qs) - 1
    cts = []
    for lane in range(len(sh.lanes)):
        for v in NB.pack_lane(sh, n // 2, lane, tokens[lane]):
            pt = torch.empty((top, n), dtype=torch.int64, device="cuda")
            ctx.encode(v, scale, top, pt)
            cts.append(ctx.seal_encrypt_symmetric(sk, pt, top, seed))
    torch.cuda.synchronize()
    x = [Ciphertext.from_device(ctx, t, scale, stream) for t in cts]
    direct = layer.forward(x, lockstep=True)       # also encodes and caches the layer's plaintexts
    stream.synchronize()
    assert _lane_digests(direct, layer.n_hid) == _want("output")
    gx = [Ciphertext.from_device(ctx, t, scale, stream) for t in cts]
    with Graph(stream) as g:
        out = layer.forward(gx, lockstep=True)
    for _ in range(2):
        g.launch()
        stream.synchronize()
        assert _lane_digests(out, layer.n_hid) == _want("output")


def test_memory_info_counts_the_engine_buffers(env):
    """Keys, LT coefficients and ciphertexts live in the engine's pool: its
    live bytes are nonzero, at most their peak and at most what it holds."""
    import torch

    import nexus_gb300 as ng
    torch.cuda.synchronize()
    m = ng.memory_info()
    assert 0 < m["pool_used"] <= m["pool_used_high"]
    assert m["pool_used"] <= m["pool_reserved"]
    ng.memory_trim()
    t = ng.memory_info()
    assert t["pool_used"] == m["pool_used"] and t["pool_reserved"] <= m["pool_reserved"]
