"""Multi-process (gloo, world size 2, CPU) test of the replica reductions bench.py uses under torchrun: the
barrier, the max of the ranks' times and the whole-job throughput (units of all ranks / slowest rank's time)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from subrosadg_gb300 import replicas
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, lr = replicas.env()
        replicas.barrier(dist)
        slowest = replicas.max_over_ranks(dist, 1.5 + rank)
        total = replicas.sum_over_ranks(dist, 1.0)
        thr = replicas.job_throughput(dist, 100.0 * (rank + 1), float(rank + 1))
        out.put((rank, w, r, lr, slowest, total, thr))
    finally:
        dist.destroy_process_group()


def test_replica_reductions_two_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, w, r, lr, slowest, total, thr in results:
        assert (w, r, lr) == (world, rank, rank)
        assert slowest == 2.5            # the slowest rank's time
        assert total == 2.0
        assert thr == (100.0 + 200.0) / 2.0  # all ranks' units / the slowest time


def test_single_process_is_the_identity():
    from subrosadg_gb300 import replicas
    assert replicas.max_over_ranks(None, 3.0) == 3.0
    assert replicas.job_throughput(None, 10.0, 2.0) == 5.0
