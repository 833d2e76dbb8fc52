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
    from magreete_gb300 import batch, _lib
    probs = sweep_problems(4, seed=5)
    cache = str(tmp_path / "tune.json")
    best = batch.autotune(probs, branch_options=(2, 4), panel_rows_options=(128, 256), cache=cache)
    assert best["branches"] in (2, 4) and best["panel_rows"] in (128, 256)
    assert len(best["candidates"]) == 4
    again = batch.autotune(probs, cache=cache)     # served from the cache
    assert again["branches"] == best["branches"]
    assert _lib.load().mgt_get_tuning(_lib.MGT_TUNE_PANEL_ROWS) == best["panel_rows"]
    _lib.load().mgt_set_tuning(_lib.MGT_TUNE_PANEL_ROWS, 256)
