"""mgt_lu_factor_static: the LU entry point that allocates nothing.

Some callers of this library cannot allocate device memory when they call
it -- a C or Fortran host that binds only the C ABI and has no allocator to
ask for the LU workspace, or a process that reserved all device memory into
its own pool up front.  For them the library keeps the LU scratch in a 1 MiB
array of its own.  This test calls that entry point through the C ABI twice
in a row (complex128 then complex64, different matrices, so the second call
runs on scratch the first one left behind) and checks that its factors and
row permutation equal those of the workspace entry point mgt_lu_factor.
"""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


def _factor_static(lib, A, dtype_code):
    from magreete_gb300 import _lib as L
    n = A.shape[0]
    perm = torch.empty(n, dtype=torch.int32, device=A.device)
    info = torch.full((2,), -99, dtype=torch.int32, device=A.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.mgt_lu_factor_static(dtype_code, ctypes.c_void_p(A.data_ptr()), n, A.stride(0),
                                  ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(info.data_ptr()), stream)
    L.check(st, "mgt_lu_factor_static")
    torch.cuda.synchronize()
    return perm, info


def test_static_scratch_lu_matches_workspace_lu():
    from magreete_gb300 import _lib as L
    from magreete_gb300 import engine as E
    lib = L.load()
    gen = torch.Generator().manual_seed(1234)
    # complex128: both entry points run the same FP64 kernels, so the factors agree to
    # rounding.  complex64: the workspace entry point may run its trailing update on the
    # tensor cores (TF32x3) while the static one stays on the FP32 pipes, so the factors
    # agree to FP32-LU accuracy (the 1e-4 bound test_lu_random uses for complex64).
    for n, dtype, code, tol in [(700, torch.complex128, L.MGT_C128, 1e-13), (1100, torch.complex64, L.MGT_C64, 1e-4)]:
        A = torch.randn(n, n, dtype=torch.complex128, generator=gen).to(dtype).cuda()
        ref = E.lu_factor(A.clone())          # workspace entry point
        A2 = A.clone()
        perm, info = _factor_static(lib, A2, code)
        assert info.tolist() == [0, 0]
        Ad = A.to(torch.complex128)
        Lm = torch.tril(A2.to(torch.complex128), -1) + torch.eye(n, dtype=torch.complex128, device="cuda")
        U = torch.triu(A2.to(torch.complex128))
        recon = (torch.linalg.norm(Lm @ U - Ad[perm.long()]) / torch.linalg.norm(Ad)).item()
        assert recon <= tol, recon
        if torch.equal(perm, ref.perm):
            err = (torch.linalg.norm(A2 - ref.lu) / torch.linalg.norm(ref.lu)).item()
            assert err <= tol, err
        # both factorisations solve the system to the same answer
        B = torch.randn(n, 3, dtype=torch.complex128, generator=gen).to(dtype).cuda()
        X = E.lu_solve(E.LUFactors(A2, perm, None, code), B).to(torch.complex128)
        Xr = E.lu_solve(ref, B).to(torch.complex128)
        assert (torch.linalg.norm(X - Xr) / torch.linalg.norm(Xr)).item() <= tol * 10
        res = (torch.linalg.norm(Ad @ X - B.to(torch.complex128)) / torch.linalg.norm(B.to(torch.complex128))).item()
        assert res < (1e-11 if dtype == torch.complex128 else 1e-3)


def test_static_scratch_rejects_oversized_n():
    from magreete_gb300 import _lib as L
    lib = L.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dummy = torch.empty(1, dtype=torch.complex64, device="cuda")
    st = lib.mgt_lu_factor_static(L.MGT_C64, ctypes.c_void_p(dummy.data_ptr()), 65537, 65537,
                                  ctypes.c_void_p(dummy.data_ptr()), ctypes.c_void_p(0), stream)
    assert st == L.MGT_ERR_UNSUPPORTED
