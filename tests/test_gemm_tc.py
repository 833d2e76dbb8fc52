"""tcgen05 TF32x3 complex trailing update against a complex128 reference."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 64), (1000, 700, 64), (257, 1029, 17),
                                   (4096, 4096, 64), (129, 33, 1)])
def test_tc_update_matches_complex128(M, N, K):
    from magreete_gb300 import engine as E
    g = torch.Generator().manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, dtype=torch.complex128, generator=g)
    B = torch.randn(K, N, dtype=torch.complex128, generator=g)
    C = torch.randn(M, N, dtype=torch.complex128, generator=g)
    A32, B32, C32 = A.to(torch.complex64), B.to(torch.complex64), C.to(torch.complex64)
    ref = C32.to(torch.complex128) - A32.to(torch.complex128) @ B32.to(torch.complex128)
    # padded leading dimension (even) for C, as the LU allocates it
    ldc = N + (N & 1) + 2
    Cbuf = torch.zeros(M, ldc, dtype=torch.complex64, device="cuda")
    Cbuf[:, :N] = C32.cuda()
    out = E.cgemm_sub(Cbuf[:, :N], A32.cuda(), B32.cuda(), tensor_cores=True)
    err = rel(out.cpu().to(torch.complex128), ref)
    # FP32-level: the complex64 rounding of the result dominates
    assert err < 2e-6, err
    assert torch.all(Cbuf[:, N:] == 0)   # padding columns keep their values
    simt = E.cgemm_sub(C32.clone().cuda(), A32.cuda(), B32.cuda(), tensor_cores=False)
    assert rel(simt.cpu().to(torch.complex128), ref) < 2e-6
