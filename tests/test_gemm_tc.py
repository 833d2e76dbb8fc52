"""tcgen05 complex trailing update (F16x2 scaled and TF32x3 split products)
against a complex128 reference."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return (torch.linalg.norm(a - b) / torch.linalg.norm(b)).item()


@pytest.fixture(params=["f16x2", "tf32x3"])
def tc_mode(request):
    """split-product scheme of the update kernel"""
    from magreete_gb300 import _lib as L
    lib = L.load()
    old = lib.mgt_get_tuning(L.MGT_TUNE_TC_PRECISION)
    lib.mgt_set_tuning(L.MGT_TUNE_TC_PRECISION, L.MGT_TC_F16X2 if request.param == "f16x2" else L.MGT_TC_TF32X3)
    yield request.param
    lib.mgt_set_tuning(L.MGT_TUNE_TC_PRECISION, old)


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (300, 200, 64), (1000, 700, 64), (257, 1029, 17),
                                   (4096, 4096, 64), (129, 33, 1), (640, 520, 128),
                                   (700, 450, 256), (333, 530, 200), (1100, 260, 129)])
def test_tc_update_matches_complex128(M, N, K, tc_mode):
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
    # FP32-level: the complex64 rounding of the result dominates for F16x2;
    # TF32x3 keeps about 21 bits per product, an error that grows like sqrt(K)
    tol = 2e-6 if tc_mode == "f16x2" else max(2e-6, 3e-7 * K ** 0.5)
    assert err < tol, err
    assert torch.all(Cbuf[:, N:] == 0)   # padding columns keep their values
    simt = E.cgemm_sub(C32.clone().cuda(), A32.cuda(), B32.cuda(), tensor_cores=False)
    assert rel(simt.cpu().to(torch.complex128), ref) < 2e-6


def test_tc_update_badly_scaled(tc_mode):
    """Rows of A and columns of B spanning 1e-15 .. 1e15: each entry of the
    update stays within FP32-level error of its own magnitude scale
    (|C| + |A| |B|), which is what the per-row / per-column power-of-two scaling
    of the fp16 split keeps."""
    from magreete_gb300 import engine as E
    M, N, K = 520, 390, 96
    g = torch.Generator().manual_seed(11)
    ra = 10.0 ** (torch.rand(M, 1, generator=g, dtype=torch.float64) * 30 - 15)
    cb = 10.0 ** (torch.rand(1, N, generator=g, dtype=torch.float64) * 30 - 15)
    A = (torch.randn(M, K, dtype=torch.complex128, generator=g) * ra).to(torch.complex64)
    B = (torch.randn(K, N, dtype=torch.complex128, generator=g) * cb).to(torch.complex64)
    C = (torch.randn(M, N, dtype=torch.complex128, generator=g) * (ra * cb)).to(torch.complex64)
    A64, B64, C64 = (x.to(torch.complex128) for x in (A, B, C))
    ref = C64 - A64 @ B64
    scale = C64.abs() + A64.abs() @ B64.abs()
    ldc = N + (N & 1) + 2
    Cbuf = torch.zeros(M, ldc, dtype=torch.complex64, device="cuda")
    Cbuf[:, :N] = C.cuda()
    out = E.cgemm_sub(Cbuf[:, :N], A.cuda(), B.cuda(), tensor_cores=True).cpu().to(torch.complex128)
    err = ((out - ref).abs() / scale).max().item()
    assert err < 1e-5, err
