"""Multi-rank host logic of the bench on CPU (gloo, world size 2): every rank
runs an independent replica (the path has no exchange step), the ranks meet
only at the barrier and at the max-over-ranks of the timed region, and the
replicas' results are each rank's own."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import time

    import torch.distributed as dist

    import bench
    from oracle import pyoracle as po
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        log_n, n = 12, 1 << 12
        qs = po.create_coeff_modulus(n, [50, 50])
        oc = po.OracleContext(log_n, qs)
        x = po.random_residues(np.random.default_rng(100 + rank), (2, 2, n), qs)  # this rank's own shard
        bench.barrier(world)
        t0 = time.perf_counter()
        y = oc.ntt(x, 0, 2)
        local = time.perf_counter() - t0 + 0.01 * rank  # ranks take different times
        slowest = bench.max_over_ranks(local, world)
        bench.barrier(world)
        out[rank] = (local, slowest, int(y.sum() % (1 << 61)), int(oc.ntt(y, 0, 2, inverse=True).sum() % (1 << 61)),
                     int(x.sum() % (1 << 61)))
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        res = dict(out)
    assert sorted(res) == [0, 1]
    slowest = max(res[r][0] for r in res)
    for r in res:
        local, mx, ysum, back, xsum = res[r]
        assert mx == pytest.approx(slowest)      # every rank reports the slowest rank's time
        assert back == xsum                      # each replica's round trip is its own data
    assert res[0][2] != res[1][2]                # independent shards, no data exchange
