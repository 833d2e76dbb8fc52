"""mgt_lu_factor_static: the LU entry point that allocates nothing.

Some callers of this library cannot allocate device memory when they call
it -- a C or Fortran host that binds only the C ABI and has no allocator to
ask for the LU workspace, or a process that reserved all device memory into
its own pool up front.  For them the library keeps the LU scratch in a 1 MiB
array of its own.  This test calls that entry point through the C ABI twice
in a row (complex128 then complex64, different matrices, so the second call
runs on scratch the first one left behind) and checks that its factors and
row permutation are bitwise those of the workspace entry point mgt_lu_factor
run with the same kernels, that a repeated call changes the device's free
memory by nothing, and that oversized systems are refused.
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


def _factor_workspace(lib, A, dtype_code, nbytes):
    """mgt_lu_factor with a workspace of exactly nbytes bytes."""
    from magreete_gb300 import _lib as L
    n = A.shape[0]
    perm = torch.empty(n, dtype=torch.int32, device=A.device)
    work = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=A.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L.check(lib.mgt_lu_factor(dtype_code, ctypes.c_void_p(A.data_ptr()), n, A.stride(0),
                              ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(work.data_ptr()), nbytes, stream),
            "mgt_lu_factor")
    torch.cuda.synchronize()
    return perm


def test_static_scratch_lu_matches_workspace_lu():
    from magreete_gb300 import _lib as L
    from magreete_gb300 import engine as E
    lib = L.load()
    gen = torch.Generator().manual_seed(1234)
    # The smallest workspace mgt_lu_factor accepts (the complex128 size: no room
    # for the tensor-core split buffers) makes it run the same kernels as the
    # static entry point, for complex64 too: the factors and the row permutation
    # must then be bitwise the same.  With its full workspace the complex64 LU
    # runs its trailing update on the tensor cores (F16x2 split products), and
    # the factors agree to FP32-LU accuracy (the 1e-4 bound test_lu_random uses
    # for complex64).
    for n, dtype, code in [(700, torch.complex128, L.MGT_C128), (1100, torch.complex64, L.MGT_C64)]:
        A = torch.randn(n, n, dtype=torch.complex128, generator=gen).to(dtype).cuda()
        base = ctypes.c_size_t()
        L.check(lib.mgt_lu_workspace_bytes(L.MGT_C128, n, ctypes.byref(base)))
        A1 = A.clone()
        perm1 = _factor_workspace(lib, A1, code, base.value)
        A2 = A.clone()
        perm, info = _factor_static(lib, A2, code)
        assert info.tolist() == [0, 0]
        assert torch.equal(perm, perm1)
        assert torch.equal(A2, A1)
        # against the full-workspace factorisation (tensor cores for complex64)
        ref = E.lu_factor(A.clone())
        tol = 1e-13 if dtype == torch.complex128 else 1e-4
        Ad = A.to(torch.complex128)
        Lm = torch.tril(A2.to(torch.complex128), -1) + torch.eye(n, dtype=torch.complex128, device="cuda")
        U = torch.triu(A2.to(torch.complex128))
        recon = (torch.linalg.norm(Lm @ U - Ad[perm.long()]) / torch.linalg.norm(Ad)).item()
        assert recon <= tol, recon
        B = torch.randn(n, 3, dtype=torch.complex128, generator=gen).to(dtype).cuda()
        X = E.lu_solve(E.LUFactors(A2, perm, None, code), B).to(torch.complex128)
        Xr = E.lu_solve(ref, B).to(torch.complex128)
        assert (torch.linalg.norm(X - Xr) / torch.linalg.norm(Xr)).item() <= tol * 10
        res = (torch.linalg.norm(Ad @ X - B.to(torch.complex128)) / torch.linalg.norm(B.to(torch.complex128))).item()
        assert res < (1e-11 if dtype == torch.complex128 else 1e-3)


def test_static_scratch_allocates_nothing():
    """A call after a warm-up one (same type and size, so no kernel is loaded
    for the first time) leaves the device's free memory unchanged."""
    from magreete_gb300 import _lib as L
    lib = L.load()
    gen = torch.Generator().manual_seed(77)
    n = 1100
    A = torch.randn(n, n, dtype=torch.complex128, generator=gen).to(torch.complex64).cuda()
    work = A.clone()
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    info = torch.zeros(2, dtype=torch.int32, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

    def call():
        work.copy_(A)
        L.check(lib.mgt_lu_factor_static(L.MGT_C64, ctypes.c_void_p(work.data_ptr()), n, n,
                                         ctypes.c_void_p(perm.data_ptr()), ctypes.c_void_p(info.data_ptr()), stream),
                "mgt_lu_factor_static")
        torch.cuda.synchronize()

    call()
    first = work.clone()
    free0, _ = torch.cuda.mem_get_info()
    call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert info.tolist() == [0, 0]
    assert torch.equal(work, first)


def test_static_scratch_rejects_oversized_n():
    from magreete_gb300 import _lib as L
    lib = L.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    dummy = torch.empty(1, dtype=torch.complex64, device="cuda")
    st = lib.mgt_lu_factor_static(L.MGT_C64, ctypes.c_void_p(dummy.data_ptr()), 65537, 65537,
                                  ctypes.c_void_p(dummy.data_ptr()), ctypes.c_void_p(0), stream)
    assert st == L.MGT_ERR_UNSUPPORTED
