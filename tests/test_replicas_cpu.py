"""The multi-GPU path runs independent replicas; its only cross-rank steps are the timing
barrier, the slowest rank's time and the summed throughput.  Two gloo ranks on CPU."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE="2", RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from neuralangelo_gb300.replicas import ReplicaGroup
    g = ReplicaGroup(backend="gloo")
    g.barrier()
    slow = g.max(1.0 + rank)                       # rank 1 is the slower one
    total = g.sum(100 * (rank + 1))
    rate = g.throughput(units=1000, seconds=0.5 * (rank + 1))
    g.barrier()
    g.close()
    q.put((rank, g.world, slow, total, rate))


def test_two_gloo_replicas_share_timing_only():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, world, slow, total, rate in res:
        assert world == 2
        assert slow == 2.0                      # the slowest rank's time on every rank
        assert total == 300.0
        assert rate == 2000 / 1.0               # both ranks' units over the slowest rank's seconds


def test_single_process_group_is_a_no_op():
    from neuralangelo_gb300.replicas import ReplicaGroup
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    g = ReplicaGroup()
    g.barrier()
    assert g.world == 1 and g.max(3.5) == 3.5 and g.throughput(10, 2.0) == 5.0
