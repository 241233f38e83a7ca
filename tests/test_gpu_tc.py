"""Tensor-core GEMM of the learned warm start (slbc_tc_gemm: tcgen05.mma
with BF16 operands staged by TMA, FP32 accumulation in TMEM) against a
plain PyTorch FP32 product of the same BF16 values.  Each product is exact
in FP32; only the summation order differs, so the tolerance is 1e-5 of the
largest entry."""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def tc(gpu):
    f = gpu.dll.slbc_tc_gemm
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    s = gpu.dll.slbc_tc_status
    s.restype = C.c_int
    return f, s


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 512), (512, 256, 1088), (384, 128, 4096)])
def test_gemm_matches_fp32(gpu, M, N, K):
    torch = pytest.importorskip("torch")
    gemm, status = tc(gpu)
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    D = torch.full((M, N + 4), float("nan"), device="cuda")
    rc = gemm(A.data_ptr(), B.data_ptr(), D.data_ptr(), M, N, K, N + 4, torch.cuda.current_stream().cuda_stream)
    assert rc == 0, gpu.dll.slbc_last_error
    assert status() == 0
    ref = A.float() @ B.float().t()
    got = D[:, :N]
    assert torch.isfinite(got).all()
    assert (got - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
    assert torch.isnan(D[:, N:]).all()  # nothing written past N


def test_gemm_rejects_bad_shapes(gpu):
    torch = pytest.importorskip("torch")
    gemm, _ = tc(gpu)
    A = torch.zeros(128, 64, device="cuda", dtype=torch.bfloat16)
    D = torch.zeros(128, 128, device="cuda")
    assert gemm(A.data_ptr(), A.data_ptr(), D.data_ptr(), 100, 128, 64, 128, None) != 0
    assert gemm(A.data_ptr(), A.data_ptr(), D.data_ptr(), 128, 128, 48, 128, None) != 0
