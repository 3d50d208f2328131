"""The tcgen05 (UMMA/TMEM) BF16 GEMM against an FP32 product of the same
BF16 operands: relative L2 <= 1e-5 (exact BF16 products, FP32 accumulation
in a different order)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 128, 256), (300, 96, 72), (1024, 256, 1152)])
def test_tc_gemm_matches_fp32_product(cdx, torch_cuda, M, N, K):
    torch = torch_cuda
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    D = torch.full((M, N), float("nan"), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    cdx.check(cdx.lib().cdx_gemm_bf16_tc(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                                          ctypes.c_void_p(D.data_ptr()), M, N, K, ctypes.c_void_p(err.data_ptr()),
                                          None))
    torch.cuda.synchronize()
    ref = A.float() @ B.float().T
    e = (torch.linalg.vector_norm(D - ref) / torch.linalg.vector_norm(ref)).item()
    print(f"tc gemm {M}x{N}x{K}: rel L2 {e:.3e}, err flag {int(err.item())}")
    assert int(err.item()) == 0
    assert e < 1e-5
