"""The multi-rank (replica) path on CPU: two gloo ranks fit disjoint shards
of the seeded scene with the oracle and reduce their counts and times the
way bench.py does; the job result equals one rank fitting both shards."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from photic_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, n, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    from oracle import oracle as O
    dist.init_process_group("gloo")
    pix0 = replicas.shard_start(rank, n)
    rrs, _ = O.generate_single(20260101, n, pix0=pix0)
    out = O.invert_batch(rrs, nthreads=1)
    fitted = float(np.sum(out[:, 9] == 0))
    fake_seconds = 1.0 + rank  # rank 1 is the slower one
    dist.barrier()
    total = replicas.sum_over_ranks(fitted, dist)
    slowest = replicas.max_over_ranks(fake_seconds, dist)
    if rank == 0:
        q.put((total, slowest, replicas.job_rate(total, slowest)))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_without_overlap():
    from oracle import oracle as O
    n = 48
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, n, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    total, slowest, rate = q.get(timeout=10)
    rrs, _ = O.generate_single(20260101, 2 * n, pix0=0)
    ref = O.invert_batch(rrs, nthreads=2)
    assert total == float(np.sum(ref[:, 9] == 0))
    assert slowest == 2.0 and rate == total / 2.0


def test_single_rank_needs_no_process_group():
    assert replicas.max_over_ranks(3.0) == 3.0
    assert replicas.sum_over_ranks(5.0) == 5.0
    assert replicas.shard_start(3, 100) == 300
    with pytest.raises(ValueError):
        replicas.job_rate(1.0, 0.0)
