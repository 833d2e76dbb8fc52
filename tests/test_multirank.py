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


@pytest.mark.timeout(300)
def test_reference_arm_rank0_prints_contract_line(capsys):
    """Rank 0 of the reference arm prints one JSON line with the bench keys
    (the oracle port's rate; a tiny calibration budget keeps this short)."""
    import json
    import bench

    class A:
        steps, warmup, requests, cpu_budget, gpus = 1, 3, 2, 0.01, 1
    bench.run_reference(A, rank=0, world=1)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["unit"] == "solves/s"
    for key in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["vs_baseline"] is None and d["higher_is_better"] is True and d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_bench_names_are_all_defined():
    """Every name bench.py loads at module level or in a function is bound
    somewhere in it (a removed helper would otherwise surface only in a full
    GPU run)."""
    import ast
    import builtins
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "bench.py")).read()
    tree = ast.parse(src)
    bound = set(dir(builtins)) | {"__file__"}
    for node in ast.walk(tree):
        if isinstance(node, (ast.FunctionDef, ast.AsyncFunctionDef, ast.ClassDef)):
            bound.add(node.name)
        elif isinstance(node, ast.Name) and isinstance(node.ctx, (ast.Store, ast.Del)):
            bound.add(node.id)
        elif isinstance(node, (ast.Import, ast.ImportFrom)):
            bound.update((a.asname or a.name).split(".")[0] for a in node.names)
        elif isinstance(node, ast.arg):
            bound.add(node.arg)
        elif isinstance(node, ast.ExceptHandler) and node.name:
            bound.add(node.name)
    used = {n.id for n in ast.walk(tree) if isinstance(n, ast.Name) and isinstance(n.ctx, ast.Load)}
    assert not (used - bound), sorted(used - bound)


def test_update_roofline_bound_follows_k():
    """The trailing update's roofline entry: a K = 128 window (16 B of C per
    64 flops) is HBM-bound, a K = 256 window tensor-bound (three F16 split
    products per flop against bf16 / 3); frac = roof time / measured time."""
    import bench
    hbm, bf16 = 6681.8, 1913.9
    M = N = 10000

    def window(K, ms):
        return 1, ms, 8.0 * M * N * K, 8.0 * (2 * M * N + K * (M + N))

    n, ms, fl, by = window(128, 0.5)
    r = bench.update_roofline(n, ms, fl, by, hbm, bf16, "measured")
    assert r["bound"] == "hbm" and r["unit"] == "GB/s" and r["peak"] == hbm
    assert r["frac"] == pytest.approx(by / (hbm * 1e9) / (ms * 1e-3))
    assert r["achieved"] == pytest.approx(by / (ms * 1e-3) / 1e9)
    n, ms, fl, by = window(256, 0.5)
    r = bench.update_roofline(n, ms, fl, by, hbm, bf16, "measured")
    assert r["bound"] == "tensor" and r["unit"] == "TFLOP/s" and r["peak"] == pytest.approx(bf16 / 3)
    assert r["frac"] == pytest.approx(3 * fl / (bf16 * 1e12) / (ms * 1e-3))
    assert r["tensor_frac"] == pytest.approx(r["frac"])
    # windows of both kinds together: the larger of the two roof-time totals decides
    # (here one K = 128 and one K = 256 window: HBM 0.488 ms against tensor 0.482 ms)
    a, b = window(128, 0.5), window(256, 0.5)
    fl, by = a[2] + b[2], a[3] + b[3]
    t_hbm, t_tc = by / (hbm * 1e9), 3 * fl / (bf16 * 1e12)
    r = bench.update_roofline(2, 1.0, fl, by, hbm, bf16, "measured")
    assert r["bound"] == ("tensor" if t_tc >= t_hbm else "hbm")
    assert r["frac"] == pytest.approx(max(t_hbm, t_tc) / 1e-3)
    assert bench.update_roofline(0, 0.0, 0.0, 0.0, hbm, bf16, "measured")["frac"] is None
