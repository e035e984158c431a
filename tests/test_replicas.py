"""CPU test of the multi-rank path (world_size 2, gloo): sharding and the timing reduction."""

import os
import socket

import torch.multiprocessing as mp

from bitgen_gb300 import replicas


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, size, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(size), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    replicas.init("gloo")
    items = list(range(11))
    mine = replicas.shard(items, rank, size)
    replicas.barrier()
    got = replicas.max_over_ranks([1.0 + rank, 5.0 - rank])
    q.put((rank, mine, got))


def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict((r, (m, g)) for r, m, g in (q.get(timeout=120) for _ in procs))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(res[0][0] + res[1][0]) == list(range(11))
    assert res[0][1] == res[1][1] == [2.0, 5.0]
