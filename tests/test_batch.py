"""Batched sweep: one CUDA graph for many uneven solves; replays reproduce the eager results."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def sweep_problems(count=6, seed=21):
    from magreete_gb300 import workloads as W
    import numpy as np
    rng = np.random.default_rng(seed)
    probs = []
    for i in range(count):
        N = int(rng.integers(150, 900))
        if i % 2 == 0:
            probs.append(W.disk_problem(N, 1000 + i, float(rng.uniform(5, 30)), n_angles=16))
        else:
            probs.append(W.cube_problem(N // 2, 2000 + i, float(rng.uniform(3, 8)), n_dirs=8))
    return probs


def test_graph_replay_matches_eager():
    from magreete_gb300 import batch, serve
    probs = sweep_problems()
    sw = batch.BatchedSweep(probs, branches=3)
    sw.warmup()
    sw.capture()
    for _ in range(2):   # replays must not see the previous run's records or flags
        extra, res = sw.replay()
        assert max(res) <= 1e-10
        for p, X in zip(probs, sw.solutions()):
            ref = serve.solve_problem(p, "mixed").Ek
            assert rel(X, ref) < 1e-8


def test_autotune_picks_and_caches(tmp_path):
    """The autotuner times every candidate, caches the fastest per size
    bucket, and leaves the library's process-wide tuning as it was."""
    from magreete_gb300 import batch, _lib
    lib = _lib.load()
    before = [lib.mgt_get_tuning(k) for k in range(1, 11)]
    probs = sweep_problems(4, seed=5)
    cache = str(tmp_path / "tune.json")
    best = batch.autotune(probs, branch_options=(2, 4), pivoting_options=("tile", "partial"), outer_options=(128,),
                          cache=cache)
    assert best["branches"] in (2, 4) and best["pivoting"] in ("tile", "partial") and best["outer_block"] == 128
    assert len(best["candidates"]) == 4
    again = batch.autotune(probs, cache=cache)     # served from the cache
    assert {k: again[k] for k in ("branches", "pivoting", "outer_block")} == \
        {k: best[k] for k in ("branches", "pivoting", "outer_block")}
    assert [lib.mgt_get_tuning(k) for k in range(1, 11)] == before


def test_partial_pivoting_graph_matches_eager():
    """Graph replays of partially pivoted (LAPACK-order) factorisations."""
    from magreete_gb300 import batch, serve
    probs = sweep_problems(4, seed=9)
    sw = batch.BatchedSweep(probs, branches=2, pivoting="partial")
    sw.warmup()
    sw.capture()
    extra, res = sw.replay()
    assert max(res) <= 1e-10
    for p, X in zip(probs, sw.solutions()):
        assert rel(X, serve.solve_problem(p, "mixed").Ek) < 1e-8
