"""Replica mode of the multi-GPU path, exercised on CPU with two gloo ranks.

Each rank loads its own plasma with its replica seed (host loader of the product library,
no GPU needed), the ranks check that their inputs differ, and the timing/work reduction
gives max(seconds) and sum(units).
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import numpy as np
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import qpad_gb300 as Q
        from qpad_gb300.replicas import reduce_timing, replica_seed
        seed = replica_seed(1, rank)
        x, p, g, ps, q_ = Q.load_plasma(32, 0.05, seed, 2, 1, 8, uth=(1e-2, 1e-2, 1e-2))
        checksum = torch.tensor([float(np.sum(p[:, 0]))], dtype=torch.float64)
        gathered = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
        dist.all_gather(gathered, checksum)
        sec, units = reduce_timing(1.0 + rank, 100.0 * (rank + 1), dist)
        q.put((rank, seed, [float(t.item()) for t in gathered], sec, units))
    finally:
        dist.destroy_process_group()


def test_two_replicas_reduce_over_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    out.sort()
    (r0, s0, g0, sec0, u0), (r1, s1, g1, sec1, u1) = out
    assert s0 != s1
    assert g0 == g1 and g0[0] != g0[1]          # replicas draw different momenta
    assert sec0 == sec1 == 2.0                  # max over ranks
    assert u0 == u1 == 300.0                    # sum over ranks


def test_reduce_timing_without_group():
    from qpad_gb300.replicas import reduce_timing, replica_seed
    assert reduce_timing(1.5, 10.0) == (1.5, 10.0)
    assert replica_seed(5, 0) == 5 and replica_seed(5, 2) != 5
