"""Replica logic of the multi-GPU path, with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from onegraph_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, lr = replicas.rank_info()
    mine = replicas.slice_queries(list(range(32)), r, w)
    replicas.barrier(w)
    slowest = replicas.max_over_ranks(1.0 + r, w, device="cpu")  # rank 1 is slower
    q.put((r, mine, slowest, replicas.whole_job_rate(len(mine), w, slowest)))
    dist.destroy_process_group()


def test_two_gloo_replicas_split_queries_and_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, q0, s0, rate0), (r1, q1, s1, rate1) = out
    assert sorted(q0 + q1) == list(range(32)) and not set(q0) & set(q1)
    assert s0 == s1 == 2.0  # both ranks see the slowest time
    assert rate0 == rate1 == 32 / 2.0


def test_single_rank_defaults():
    assert replicas.slice_queries([1, 2, 3], 0, 1) == [1, 2, 3]
    assert replicas.max_over_ranks(3.5, 1) == 3.5
