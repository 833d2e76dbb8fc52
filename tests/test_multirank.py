"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The path does not shard a single solve: N GPUs run N independent replicas,
each serving its own windows of the request stream.  What the ranks share is
host logic -- per-rank stream seeds, the barrier around the timed region, the
max-over-ranks time and the whole-job request count -- and the reference arm,
which runs on rank 0 only.  These run here as two gloo processes.
"""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        assert (r, w, local) == (rank, world, rank)
        wins = bench.windows(1, 1, 4, rank)
        first = [(p.kind, p.N, p.seed) for p in wins[1]]
        dist.barrier()
        slowest = bench.max_over_ranks(0.5 + rank, world, torch.device("cpu"))
        gathered = [None] * world
        dist.all_gather_object(gathered, first)
        q.put((rank, slowest, gathered))
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    # every rank sees the slowest replica's time
    assert [o[1] for o in out] == [1.5, 1.5]
    # ranks serve different windows of the stream (rank-dependent seeds), and agree on who has what
    g0, g1 = out[0][2], out[1][2]
    assert g0 == g1
    assert g0[0] != g0[1]


def test_single_rank_max_is_identity():
    import bench
    assert bench.max_over_ranks(3.25, 1, torch.device("cpu")) == 3.25


def test_reference_arm_other_ranks_exit_without_work(capsys):
    import bench

    class A:
        steps, warmup, requests, cpu_budget, gpus = 1, 3, 2, 1.0, 2
    bench.run_reference(A, rank=1, world=2)
    assert capsys.readouterr().out == ""
