"""The tensor-core residual (digit-split / Ozaki scheme, csrc/residual_tc.cu).

R = B - M X with M in double-float form is what iterative refinement
(Transmission2D.py:230 / Transmission3D.py:205 replaced by a complex64 LU
plus refinement) needs to complex128 accuracy.  The tensor-core kernel is
held to an FP64 product of the same double-float matrix:
  * entry-wise within n 2^-48 of |M| |X| (the double-float kernel's bound),
  * and in Frobenius norm within 1e-13 of ||B|| on a system-like matrix,
across ragged shapes: rows and K off the 128 / 32 tiles, 1, 33 and 65
right-hand sides (one, two and three column tiles), K split across CTAs or
not.  The double-float kernel (selected by a workspace too small for the
tensor-core buffers) is checked beside it.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _system(n_pts, kind, seed):
    from magreete_gb300 import engine as E
    gen = torch.Generator().manual_seed(seed)
    dim = 2 if kind.startswith("2d") else 3
    pts = (torch.rand(n_pts, dim, dtype=torch.float64, generator=gen) * (8.0 if dim == 2 else 2.0)).cuda()
    M, Mdf = E.assemble_system(kind, pts, 2 * np.pi * 3.0, 0.05 + 0.01j, 0.02 - 0.003j, ("c128", "cdf"))
    return M, Mdf, gen


def _df_matrix(Mdf):
    """The complex128 value of the double-float matrix (hi + lo)."""
    v = Mdf.double()
    return torch.complex(v[..., 0] + v[..., 1], v[..., 2] + v[..., 3])


def _residual_with(Mdf, X, B, nbytes):
    from magreete_gb300 import _lib as L
    lib = L.load()
    n, R = B.shape
    work = torch.empty(max(nbytes, 256), dtype=torch.uint8, device="cuda")
    out = torch.empty_like(B)
    L.check(lib.mgt_residual(ctypes.c_void_p(Mdf.data_ptr()), n, n, ctypes.c_void_p(X.data_ptr()), R,
                             ctypes.c_void_p(B.data_ptr()), R, ctypes.c_void_p(out.data_ptr()), R, R,
                             ctypes.c_void_p(work.data_ptr()), work.numel(),
                             ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "mgt_residual")
    return out


@pytest.mark.parametrize("kind,n_pts,R", [("2d_vector", 700, 1), ("2d_vector", 1537, 33), ("3d_vector", 411, 65),
                                          ("3d_scalar", 2999, 5), ("2d_scalar", 4100, 64)])
def test_tc_residual_matches_fp64(kind, n_pts, R):
    from magreete_gb300 import engine as E
    M, Mdf, gen = _system(n_pts, kind, n_pts + R)
    n = M.shape[0]
    Mv = _df_matrix(Mdf)
    X = torch.randn(n, R, dtype=torch.complex128, generator=gen).cuda()
    # a right-hand side close to M X (a residual with cancellation, as in refinement)
    B = (Mv @ X) * (1 + 1e-9) + 1e-8 * torch.randn(n, R, dtype=torch.complex128, generator=gen).cuda()
    ref = B - Mv @ X
    got = E.residual(Mdf, X, B)          # queried workspace: the tensor-core kernel
    bound = n * 2.0 ** -48 * (Mv.abs() @ X.abs())
    assert torch.all((got - ref).abs() <= bound), float(((got - ref).abs() / bound).max())
    rel = (torch.linalg.norm(got - ref) / torch.linalg.norm(B)).item()
    assert rel < 1e-13, rel
    df = _residual_with(Mdf, X, B, n * R * 16)   # double-float kernel
    assert torch.all((df - ref).abs() <= bound)


def test_tc_residual_zero_columns_and_rows():
    """A zero right-hand-side column and a zero X column give exact results
    there (their scales fall back to 1)."""
    from magreete_gb300 import engine as E
    M, Mdf, gen = _system(300, "2d_vector", 3)
    n = M.shape[0]
    Mv = _df_matrix(Mdf)
    X = torch.randn(n, 4, dtype=torch.complex128, generator=gen).cuda()
    X[:, 2] = 0
    B = torch.randn(n, 4, dtype=torch.complex128, generator=gen).cuda()
    got = E.residual(Mdf, X, B)
    assert torch.equal(got[:, 2], B[:, 2])
    ref = B - Mv @ X
    assert (torch.linalg.norm(got - ref) / torch.linalg.norm(B)).item() < 1e-13


def test_refinement_uses_tc_residual_and_converges():
    """A refined solve of order 6000 with 40 right-hand sides reaches 1e-10
    with the tensor-core residual, and agrees with the FP64 solve."""
    from magreete_gb300 import engine as E
    from magreete_gb300 import workloads as W
    prob = W.disk_problem(3000, 21, 12.0, n_angles=40)
    pts = prob.points.cuda()
    from magreete_gb300 import selfterm, serve
    shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
    E0s, _ = serve.incident_fields(prob, pts, prob.detectors.cuda())
    Bv = E0s.reshape(prob.n, -1).contiguous()
    coef = prob.alpha * prob.k0 ** 2
    st = {}
    X = E.solve_system(prob.kind, pts, prob.k0, coef, shift, Bv, "mixed", stats=st)
    assert st["rel_residual"] <= 1e-10
    X64 = E.solve_system(prob.kind, pts, prob.k0, coef, shift, Bv, "fp64")
    assert (torch.linalg.norm(X - X64) / torch.linalg.norm(X64)).item() < 1e-8


def test_prepared_operator_matches_one_shot_residual():
    """mgt_residual_prepare once, mgt_residual_apply for several X (fewer
    columns than prepared for, too): bit-identical to mgt_residual."""
    from magreete_gb300 import engine as E
    M, Mdf, gen = _system(900, "3d_vector", 11)
    n = M.shape[0]
    op = E.ResidualOperator(Mdf, 40)
    for R in (40, 7):
        X = torch.randn(n, R, dtype=torch.complex128, generator=gen).cuda()
        B = torch.randn(n, R, dtype=torch.complex128, generator=gen).cuda()
        assert torch.equal(op(X, B), E.residual(Mdf, X, B))
    with pytest.raises(ValueError):
        op(X[:, :1].repeat(1, 41), B[:, :1].repeat(1, 41))


def test_refinement_from_prepared_digits():
    """mgt_refine_prepare, then the double-float matrix freed: refined solves
    through the prepared digits give the same fields as solves from the
    matrix (bitwise for one block of columns; wider right-hand sides in
    column blocks within 1e-9)."""
    from magreete_gb300 import engine as E
    from magreete_gb300 import selfterm, serve
    from magreete_gb300 import workloads as W
    prob = W.disk_problem(1500, 31, 14.0, n_angles=40)
    pts = prob.points.cuda()
    shift = selfterm.diagonal_shift(prob.kind, prob.k0, prob.alpha, prob.radius)
    coef = prob.alpha * prob.k0 ** 2
    Mdf, M32 = E.assemble_system(prob.kind, pts, prob.k0, coef, shift, ("cdf", "c64"))
    E0s, _ = serve.incident_fields(prob, pts, prob.detectors.cuda())
    B = E0s.reshape(prob.n, -1).contiguous()
    f = E.lu_factor(M32.clone(), pivoting="partial")
    X_ref, it_ref, rr_ref = E.solve_refined(Mdf, f, B)
    ctx = E.RefineContext(Mdf.clone(), B.shape[1])
    X1, it1, rr1 = E.solve_refined(ctx, f, B)
    # the norms are sums in atomic order: equal to rounding
    assert torch.equal(X1, X_ref) and it1 == it_ref and rr1 == pytest.approx(rr_ref, rel=1e-12)
    narrow = E.RefineContext(Mdf, 16)
    del Mdf
    X2, it2, rr2 = E.solve_refined(narrow, f, B)
    assert rr2 <= 1e-10
    assert (torch.linalg.norm(X2 - X_ref) / torch.linalg.norm(X_ref)).item() < 1e-9
