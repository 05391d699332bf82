"""Multi-rank reactor sharding on CPU (gloo, world size 2): every reactor is integrated by
exactly one rank and the gathered result equals the single-process one."""
import os
import socket

import numpy as np
import pytest

from conftest import DATA, ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, q):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    from cantera_gb300.sharding import gather_shards, max_over_ranks, shard_range
    from oracle import pyoracle as po
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = po.Mech(os.path.join(DATA, "h2o2.yaml"), "ohmech")
        rng = np.random.default_rng(5)
        T0 = rng.uniform(1000.0, 1300.0, n)
        P = np.full(n, 101325.0)
        Y0 = np.array([m.equivalence_ratio(phi, "H2:1", "O2:1, N2:3.76") for phi in rng.uniform(0.7, 1.3, n)])
        lo, hi = shard_range(n, rank, world)
        o = po.opts(rtol=1e-8, atol=1e-15)
        T, Y, st, _ = m.advance_batch(T0[lo:hi], P[lo:hi], Y0[lo:hi], 2e-4, o, threads=1)
        Tall = gather_shards(T, n, dist)
        Yall = gather_shards(Y, n, dist, axis=0)
        idx = gather_shards(np.arange(lo, hi), n, dist)
        tmax = max_over_ranks(float(rank + 1), dist)
        if rank == 0:
            q.put((Tall, Yall, idx, tmax))
    finally:
        dist.destroy_process_group()


def test_shard_ranges_partition():
    from cantera_gb300.sharding import shard_range
    for n in (0, 1, 7, 65536):
        for w in (1, 2, 3, 8):
            got = [shard_range(n, r, w) for r in range(w)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(got, got[1:]))
            assert max(h - l for l, h in got) - min(h - l for l, h in got) <= 1
    with pytest.raises(ValueError):
        shard_range(4, 2, 2)


def test_two_rank_gloo_matches_single_process():
    import torch.multiprocessing as mp
    from oracle import pyoracle as po
    n, world = 6, 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    Tall, Yall, idx, tmax = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    np.testing.assert_array_equal(idx, np.arange(n))
    assert tmax == 2.0
    # single process, same inputs
    m = po.Mech(os.path.join(DATA, "h2o2.yaml"), "ohmech")
    rng = np.random.default_rng(5)
    T0 = rng.uniform(1000.0, 1300.0, n)
    P = np.full(n, 101325.0)
    Y0 = np.array([m.equivalence_ratio(phi, "H2:1", "O2:1, N2:3.76") for phi in rng.uniform(0.7, 1.3, n)])
    T, Y, st, _ = m.advance_batch(T0, P, Y0, 2e-4, po.opts(rtol=1e-8, atol=1e-15), threads=1)
    np.testing.assert_array_equal(Tall, T)
    np.testing.assert_array_equal(Yall, Y)
