"""Multi-process path on the CPU: world size 2 over gloo (127.0.0.1).

The quadrature of a cell is split into node ranges (one per rank); the Fermi bisection sums
the per-rank electron counts with one scalar all-reduce per step.  The sharded result must
equal the single-process oracle (sqo_fermi_density_energy uses the same bracket and rule).
"""
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


def _worker(rank, world, port, lam, w, beta, ne, out):
    import torch.distributed as dist
    from sqminiapp_gb300 import sharding
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        b, e = sharding.node_range(lam.shape[0], rank, world)
        my_l, my_w = lam[b:e], w[b:e]
        s, mn, mx = sharding.torch_reducers()
        lf, it = sharding.fermi_level(sharding.numpy_count(my_l, my_w, beta), my_l.min(),
                                      my_l.max(), ne, s, mn, mx)
        out[rank] = lf
    finally:
        dist.destroy_process_group()


def test_node_ranges_partition():
    from sqminiapp_gb300.sharding import node_range
    for n in (1, 7, 3366, 39304):
        for world in (1, 2, 3, 8):
            ranges = [node_range(n, r, world) for r in range(world)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(world - 1))


def test_sharded_fermi_level_matches_single_process(oracle_mod):
    rng = np.random.default_rng(5)
    lam = rng.uniform(-1.0, 4.0, (501, 10))
    w = rng.dirichlet(np.ones(10), 501)
    beta, ne = 50.0, 300.0
    ref = oracle_mod.fermi_density_energy(lam, w, beta, ne, 1.0)
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, lam, w, beta, ne, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out[0] == out[1]
    assert out[0] == pytest.approx(ref["lambda_f"], abs=1e-11)
