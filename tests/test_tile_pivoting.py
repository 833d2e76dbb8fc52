"""Tile pivoting (MGT_PIVOT_TILE) for the mixed method's complex64 LU.

Each 64-column panel picks its pivots among the rows of its diagonal tile
and solves the rows below against the tile's U, so no panel exchanges
anything between CTAs.  The factors are exact factors of a row permutation
(P A = L U to FP32 rounding, rows moving only within their 64-row tile);
the solution's accuracy comes from the refinement, which the mixed method
always runs and which falls back to partial pivoting (LAPACK's, the
reference's ?gesv) when it cannot use the tile-pivoted factors.
"""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


def _system64(kind, N, seed, k):
    from magreete_gb300 import engine as E
    from magreete_gb300 import selfterm
    from magreete_gb300 import workloads as W
    prob = W.disk_problem(N, seed, k, n_angles=8) if kind == "2d" else W.cube_problem(N, seed, k, n_dirs=4)
    pts = prob.points.cuda()
    coef = prob.alpha * prob.k0 ** 2
    shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
    Mdf, M32 = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("cdf", "c64"))
    return prob, pts, coef, shift, Mdf, M32


@pytest.mark.parametrize("kind,N,k", [("2d", 350, 10.0), ("2d", 1500, 20.0), ("3d", 1700, 10.0), ("3d", 4000, 10.0)])
def test_tile_lu_is_a_factorisation(kind, N, k):
    """P A = L U (to FP32 rounding times n and the growth of U) with rows
    permuted only within their tile, for both outer block widths and the
    in-order / overlapped schedules."""
    from magreete_gb300 import _lib as L
    from magreete_gb300 import engine as E
    prob, pts, coef, shift, Mdf, M32 = _system64(kind, N, 5, k)
    n = prob.n
    A = M32.clone().to(torch.complex128)
    for ob, la in [(128, 1), (128, 0), (64, 1)]:
        f = E.lu_factor(M32.clone(), check_singular=False, options=L.LuOptions(pivoting=L.MGT_PIVOT_TILE,
                                                                                outer_block=ob, lookahead=la))
        assert E.lu_info(f) == (0, 0)
        perm = f.perm.long()
        idx = torch.arange(n, device="cuda")
        assert torch.equal(perm // 64, idx // 64)
        assert torch.equal(torch.sort(perm).values, idx)
        LU = f.lu.to(torch.complex128)
        Lm = torch.tril(LU, -1) + torch.eye(n, dtype=torch.complex128, device="cuda")
        U = torch.triu(LU)
        # backward error of an FP32 LU grows with n and with the growth of U
        # (not bounded by pivoting from outside the tile)
        growth = max(1.0, (U.abs().max() / A.abs().max()).item())
        assert rel(Lm @ U, A[perm]) < 5e-8 * n * growth, growth


@pytest.mark.parametrize("kind,N,k", [("2d", 1500, 20.0), ("3d", 1700, 10.0)])
def test_tile_lu_paired_blocks(kind, N, k):
    """Paired 128-wide blocks (the columns right of a pair take one K = 256
    update; forced at these orders by lowering MGT_TUNE_WIDE_UPDATE): the same
    factorisation property, and refined solves that agree with those of the
    unpaired schedule."""
    from magreete_gb300 import _lib as L
    from magreete_gb300 import engine as E
    from magreete_gb300 import serve
    lib = L.load()
    prob, pts, coef, shift, Mdf, M32 = _system64(kind, N, 9, k)
    n = prob.n
    A = M32.clone().to(torch.complex128)
    opts = L.LuOptions(pivoting=L.MGT_PIVOT_TILE, outer_block=128, lookahead=1)
    old = lib.mgt_get_tuning(L.MGT_TUNE_WIDE_UPDATE)
    try:
        lib.mgt_set_tuning(L.MGT_TUNE_WIDE_UPDATE, 256)
        fw = E.lu_factor(M32.clone(), check_singular=False, options=opts)
        lib.mgt_set_tuning(L.MGT_TUNE_WIDE_UPDATE, 0)
        f1 = E.lu_factor(M32.clone(), check_singular=False, options=opts)
    finally:
        lib.mgt_set_tuning(L.MGT_TUNE_WIDE_UPDATE, old)
    assert E.lu_info(fw) == (0, 0)
    perm = fw.perm.long()
    idx = torch.arange(n, device="cuda")
    assert torch.equal(perm // 64, idx // 64)
    assert torch.equal(torch.sort(perm).values, idx)
    LU = fw.lu.to(torch.complex128)
    Lm = torch.tril(LU, -1) + torch.eye(n, dtype=torch.complex128, device="cuda")
    U = torch.triu(LU)
    growth = max(1.0, (U.abs().max() / A.abs().max()).item())
    assert rel(Lm @ U, A[perm]) < 5e-8 * n * growth, growth
    # the two schedules differ only in the rounding of the updates (which can
    # flip a near-tie between two pivot candidates)
    if torch.equal(fw.perm, f1.perm):
        assert rel(fw.lu, f1.lu) < 1e-4
    E0s, _ = serve.incident_fields(prob, pts, prob.detectors.cuda())
    B = E0s.reshape(n, -1).contiguous()
    Xw, it_w, rr_w = E.solve_refined(Mdf, fw, B)
    X1, it_1, rr_1 = E.solve_refined(Mdf, f1, B)
    assert rr_w <= 1e-10 and rr_1 <= 1e-10
    assert rel(Xw, X1) < 1e-9


@pytest.mark.parametrize("kind,N,k", [("2d", 1000, 20.0), ("3d", 1400, 10.0)])
def test_tile_pivoted_refined_solve_matches_partial(kind, N, k):
    """Refined solves from tile-pivoted and partially pivoted factors agree
    with each other and with the oracle."""
    from magreete_gb300 import engine as E
    prob, pts, coef, shift, Mdf, M32 = _system64(kind, N, 7, k)
    from magreete_gb300 import serve
    E0s, _ = serve.incident_fields(prob, pts, prob.detectors.cuda())
    B = E0s.reshape(prob.n, -1).contiguous()
    ft = E.lu_factor(M32.clone(), pivoting="tile")
    fp = E.lu_factor(M32.clone(), pivoting="partial")
    Xt, it_t, rr_t = E.solve_refined(Mdf, ft, B)
    Xp, it_p, rr_p = E.solve_refined(Mdf, fp, B)
    assert rr_t <= 1e-10 and rr_p <= 1e-10
    assert it_t <= it_p + 1
    assert rel(Xt, Xp) < 1e-9
    ref = O.solve(prob.kind, prob.points.numpy(), prob.k0, prob.alpha, prob.radius, E0s.cpu().numpy())
    assert rel(Xt.cpu(), torch.from_numpy(ref)) < 1e-8


def _df_pack(M):
    """(n, n, 4) float32 double-float form of a complex128 matrix."""
    hr = M.real.float()
    hi = M.imag.float()
    return torch.stack([hr, (M.real - hr.double()).float(), hi, (M.imag - hi.double()).float()], -1).contiguous()


def test_zero_tile_pivot_falls_back_to_partial():
    """A nonsingular matrix whose first tile column is zero within the tile:
    the tile LU reports the zero pivot (info = 1) and the mixed method refactors
    with partial pivoting and solves to 1e-10."""
    from magreete_gb300 import engine as E
    g = torch.Generator().manual_seed(3)
    n = 300
    M = torch.randn(n, n, dtype=torch.complex128, generator=g) + 30 * torch.eye(n, dtype=torch.complex128)
    M[:64, 0] = 0
    M = M.cuda()
    B = torch.randn(n, 3, dtype=torch.complex128, generator=g).cuda()
    ft = E.lu_factor(M.to(torch.complex64), check_singular=False, pivoting="tile")
    assert E.lu_info(ft)[1] == 1
    fresh = lambda: M.to(torch.complex64)
    f, X, it, rr = E.mixed_factor_solve(_df_pack(M), M.to(torch.complex64), B, fresh)
    assert f.pivoting == "partial" and rr <= 1e-10
    assert rel(X, torch.linalg.solve(M, B)) < 1e-9


def test_refinement_failure_falls_back_to_partial():
    """Tile pivots that are tiny (not zero) make useless factors: the
    refinement stalls, and the mixed method refactors with partial pivoting."""
    from magreete_gb300 import engine as E
    g = torch.Generator().manual_seed(4)
    n = 256
    M = torch.randn(n, n, dtype=torch.complex128, generator=g) + 20 * torch.eye(n, dtype=torch.complex128)
    M[:64, :64] *= 1e-30
    M = M.cuda()
    B = torch.randn(n, 2, dtype=torch.complex128, generator=g).cuda()
    fresh = lambda: M.to(torch.complex64)
    f, X, it, rr = E.mixed_factor_solve(_df_pack(M), M.to(torch.complex64), B, fresh)
    assert f.pivoting == "partial" and rr <= 1e-10
    assert rel(X, torch.linalg.solve(M, B)) < 1e-8


def test_options_are_per_call():
    """Per-call options leave the process-wide tuning untouched, and bad
    options are refused."""
    from magreete_gb300 import _lib as L
    lib = L.load()
    before = [lib.mgt_get_tuning(k) for k in range(1, 11)]
    A = torch.randn(200, 200, dtype=torch.complex64, device="cuda") + 20 * torch.eye(200, device="cuda")
    from magreete_gb300 import engine as E
    E.lu_factor(A.clone(), options=L.LuOptions(pivoting=L.MGT_PIVOT_TILE, panel_rows=64, cooperative=0,
                                              lookahead=0, outer_block=64))
    assert [lib.mgt_get_tuning(k) for k in range(1, 11)] == before
    nb = ctypes.c_size_t()
    L.check(lib.mgt_lu_workspace_bytes(L.MGT_C64, 200, ctypes.byref(nb)))
    work = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    perm = torch.empty(200, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for bad in (L.LuOptions(pivoting=7), L.LuOptions(outer_block=96), L.LuOptions(panel_rows=8)):
        st = lib.mgt_lu_factor_ex(L.MGT_C64, ctypes.c_void_p(A.data_ptr()), 200, 200, ctypes.c_void_p(perm.data_ptr()),
                                  ctypes.c_void_p(work.data_ptr()), nb.value, ctypes.byref(bad), stream)
        assert st == L.MGT_ERR_ARG
    A64 = A.to(torch.complex128)
    st = lib.mgt_lu_factor_ex(L.MGT_C128, ctypes.c_void_p(A64.data_ptr()), 200, 200, ctypes.c_void_p(perm.data_ptr()),
                              ctypes.c_void_p(work.data_ptr()), nb.value,
                              ctypes.byref(L.LuOptions(pivoting=L.MGT_PIVOT_TILE)), stream)
    assert st == L.MGT_ERR_UNSUPPORTED


def test_batched_sweep_tile_vs_oracle():
    """A captured group of uneven instances with tile pivoting: every
    instance reaches 1e-10 and matches the oracle."""
    from magreete_gb300 import batch
    from magreete_gb300 import workloads as W
    probs = [W.disk_problem(N, 300 + i, kl, n_angles=6) for i, (N, kl) in enumerate([(400, 8.0), (900, 15.0),
                                                                                      (650, 25.0), (1200, 12.0)])]
    sw = batch.BatchedSweep(probs, branches=4, pivoting="tile")
    sw.warmup()
    sw.capture()
    extra, res = sw.replay()
    assert max(res) <= 1e-10
    for p, X in zip(probs, sw.solutions()):
        E0 = O.source_2d(p.kind, "plane", p.points.numpy(), p.k0, p.thetas, 0.2)
        ref = O.solve(p.kind, p.points.numpy(), p.k0, p.alpha, p.radius, E0)
        assert rel(X.cpu(), torch.from_numpy(ref)) < 1e-8
