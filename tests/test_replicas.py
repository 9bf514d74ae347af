"""Replicas across ranks (the multi-GPU mode of the bench: independent flakes and vectors
per rank, no data-path collective). Host-side logic on CPU with two gloo ranks."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)

    class A:
        flakes, min_sites, max_sites, seed = 2, 2000, 4000, 1234
    hs, h, offsets = bench.build_workload(A, rank)
    # rank r did (r + 1) units of work in (r + 2) seconds: the job did 1 + 2 units in 3 s
    rate, t = bench.job_rate(rank + 1, rank + 2, dist)
    out.put((rank, rate, t, int(h.nnz), [x.shape[0] for x in hs]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas_rate_and_independent_workloads():
    import multiprocessing as mp
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, t, nnz, sizes in res:
        assert t == 3.0 and abs(rate - 1.0) < 1e-12
    # each rank builds its own flakes (rank-dependent seeds): different systems, no exchange
    assert res[0][4] != res[1][4]


def test_job_rate_single_process():
    import bench
    assert bench.job_rate(10.0, 4.0) == (2.5, 4.0)
