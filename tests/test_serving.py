"""Serving: each result is the same alone and in the mix; HBM-budget admission."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def small_stream(n=6, seed=3):
    from magreete_gb300 import workloads as W
    probs = W.serving_stream(n, seed=seed, n_min=150, n_max=700)
    for p in probs:
        p.arrival = 0.0
    return probs


def rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_alone_equals_mix(precision):
    from magreete_gb300 import serve
    probs = small_stream()
    alone = serve.serve_sequential(probs, precision)
    with serve.Server(slots=3, precision=precision) as srv:
        futs = [srv.submit(p) for p in probs]
        mix = [f.result() for f in futs]
    for a, m in zip(alone, mix):
        assert rel(m.Ek, a.Ek) <= 1e-12
        assert rel(m.E_det, a.E_det) <= 1e-12
        if precision == "mixed":
            assert m.rel_residual <= 1e-10


def test_budget_admission_and_rejection():
    from magreete_gb300 import serve
    probs = small_stream(4, seed=9)
    biggest = max(serve.matrix_bytes(p) for p in probs)
    # a budget that holds one request at a time still serves them all
    with serve.Server(slots=3, hbm_budget=biggest) as srv:
        res = [f.result() for f in [srv.submit(p) for p in probs]]
        assert srv.in_use == 0
    assert all(r.rel_residual <= 1e-10 for r in res)
    with serve.Server(slots=2, hbm_budget=biggest // 10) as srv:
        with pytest.raises(MemoryError):
            srv.submit(probs[0]).result()


def test_factorization_reuse_for_requery():
    import dataclasses
    from magreete_gb300 import serve
    p = small_stream(1, seed=11)[0]
    q = dataclasses.replace(p)              # same geometry, same frequency, new request
    with serve.Server(slots=1, factor_cache=2) as srv:
        r1 = srv.submit(p).result()
        r2 = srv.submit(q).result()
    assert r2.reused_factorization and not r1.reused_factorization
    assert rel(r2.Ek, r1.Ek) <= 1e-12
