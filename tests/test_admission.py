"""Serving admission on CPU: arrival order, the HBM budget, cached
factorisations giving way, and shutdown (serve.Admission, the part of the
Server that decides what runs)."""
import threading
import time

import pytest

from magreete_gb300.serve import Admission


def take_in_thread(adm):
    out = []
    t = threading.Thread(target=lambda: out.append(adm.take()), daemon=True)
    t.start()
    return t, out


def test_admits_in_order_within_budget():
    adm = Admission(100)
    adm.put("a", 60)
    adm.put("b", 60)
    adm.put("c", 30)
    assert adm.take() == ("a", 60) and adm.in_use == 60
    t, out = take_in_thread(adm)
    time.sleep(0.05)
    # "b" does not fit beside "a"; "c" would, but it does not overtake "b"
    assert t.is_alive() and out == []
    adm.release(60)
    t.join(2)
    assert out == [("b", 60)] and adm.in_use == 60
    assert adm.take() == ("c", 30) and adm.in_use == 90


def test_oversize_request_rejected():
    adm = Admission(100)
    with pytest.raises(MemoryError):
        adm.put("big", 101)
    assert not adm.queue


def test_cached_objects_give_way_to_a_waiting_request():
    adm = Admission(100)
    adm.cache_put("f1", object(), 50, limit=4)
    adm.cache_put("f2", object(), 30, limit=4)
    assert adm.in_use == 80
    adm.put("r", 60)
    # only the least recently used entry has to go
    assert adm.take() == ("r", 60)
    assert adm.cache_get("f1") is None and adm.cache_get("f2") is not None
    assert adm.in_use == 90


def test_cache_limit_and_lru_order():
    adm = Admission(1000)
    objs = [object() for _ in range(3)]
    adm.cache_put("k0", objs[0], 10, limit=2)
    adm.cache_put("k1", objs[1], 20, limit=2)
    assert adm.cache_get("k0") is objs[0]          # k0 is now the most recent
    adm.cache_put("k2", objs[2], 30, limit=2)      # evicts k1
    assert adm.cache_get("k1") is None
    assert adm.cache_get("k0") is objs[0] and adm.cache_get("k2") is objs[2]
    assert adm.in_use == 40
    adm.cache_put("k2", objs[2], 35, limit=2)      # the same key again is held once
    assert adm.in_use == 45


def test_close_drains_then_stops_waiters():
    adm = Admission(100)
    adm.put("a", 10)
    adm.close()
    assert adm.take() == ("a", 10)
    assert adm.take() is None
    adm2 = Admission(100)
    t, out = take_in_thread(adm2)
    time.sleep(0.05)
    assert t.is_alive()
    adm2.close()
    t.join(2)
    assert out == [None]


def test_many_workers_never_exceed_budget():
    adm = Admission(100)
    needs = [10, 40, 70, 25, 55, 5, 90, 33] * 5
    for i, n in enumerate(needs):
        adm.put(i, n)
    adm.close()
    peak = [0]
    lock = threading.Lock()
    done = []

    def worker():
        while True:
            got = adm.take()
            if got is None:
                return
            with lock:
                peak[0] = max(peak[0], adm.in_use)
            time.sleep(0.001)
            adm.release(got[1])
            with lock:
                done.append(got[0])

    ws = [threading.Thread(target=worker) for _ in range(4)]
    for w in ws:
        w.start()
    for w in ws:
        w.join(10)
    assert sorted(done) == list(range(len(needs)))
    assert peak[0] <= 100 and adm.in_use == 0


@pytest.mark.parametrize("kind,N,R,T", [("2d_vector", 1026, 1, 360), ("2d_vector", 8000, 16, 360),
                                        ("3d_vector", 4000, 64, 1024), ("3d_vector", 14420, 64, 1024),
                                        ("3d_vector", 20000, 128, 1024)])
def test_request_estimate_covers_the_library_workspaces(kind, N, R, T):
    """serve.matrix_bytes, the HBM a request is admitted with, covers what the
    library's own workspace queries ask for at the request's peak: the
    matrix copies (24 B per entry) with the refinement workspace (the
    residual's digits, the right-hand-side blocks, the triangular solves'
    workspace) and the LU's (its tensor-core split buffers), and the
    propagation workspace.  Host-only queries: no GPU needed."""
    import ctypes
    from types import SimpleNamespace
    import torch
    from magreete_gb300 import _lib as L
    from magreete_gb300 import serve
    import os
    if not os.path.exists(L.LIB_PATH):
        pytest.skip("library not built")
    lib = L.load()
    d = 2 if kind.startswith("2d") else 3
    n = d * N

    def q(fn, *args):
        nb = ctypes.c_size_t()
        L.check(fn(*args, ctypes.byref(nb)))
        return nb.value

    prob = SimpleNamespace(kind=kind, n=n, nrhs=R, d=d, detectors=torch.zeros(T, d))
    est = serve.matrix_bytes(prob, "mixed")
    refine = q(lib.mgt_refine_workspace_bytes, n, R)
    lu = q(lib.mgt_lu_workspace_bytes, L.MGT_C64, n)
    prop = q(lib.mgt_propagate_workspace_bytes, L.KIND_CODE[kind] if hasattr(L, "KIND_CODE") else
             {"2d_vector": L.MGT_2D_VECTOR, "3d_vector": L.MGT_3D_VECTOR}[kind], T, N, R)
    assert est >= 24 * n * n + refine + lu, (est, refine, lu)
    assert est >= 8 * n * n + prop + 16 * n * R
