"""Replica sharding and the timing reduction, as two gloo ranks on CPU."""
import os
import socket

import pytest

from forceatlas2_rc_gb300.replicas import max_over_ranks, shard_graphs


def test_shard_partition_is_complete_and_balanced():
    nodes = [50, 20000, 300, 7000, 7000, 1200, 90, 15000, 64, 4096]
    edges = [4 * n for n in nodes]
    for ws in (1, 2, 3, 4):
        parts = [shard_graphs(nodes, edges, ws, r) for r in range(ws)]
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(nodes)))
        loads = [sum(nodes[i] + edges[i] for i in p) for p in parts]
        # greedy LPT: within the largest single graph of the best split
        assert max(loads) - min(loads) <= max(nodes) * 5
    with pytest.raises(ValueError):
        shard_graphs(nodes, edges, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        nodes = [100 * (k + 1) for k in range(9)]
        mine = shard_graphs(nodes, nodes, ws, rank)
        t = max_over_ranks(1.5 + rank)
        q.put((rank, mine, t))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    # each rank computed its share alone; together they cover every graph once
    assert sorted(out[0][1] + out[1][1]) == list(range(9))
    assert not set(out[0][1]) & set(out[1][1])
    # the slowest rank's time is everyone's
    assert out[0][2] == out[1][2] == 2.5
    assert max_over_ranks(3.0) == 3.0  # no process group here
