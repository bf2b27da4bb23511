"""tcgen05 BF16 GEMM (FP32 accumulation in tensor memory) against a torch fp32
reference of the same product: bf16 products are exact in fp32, so only the
summation order differs (tolerance 1e-5 relative to the row norm)."""
import ctypes

import pytest
import torch

from formura_gb300 import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 128, 192), (384, 192, 576)])
def test_tc_gemm_bf16(cuda_device, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.full((M, N), float("nan"), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = _lib.lib().fm_tc_gemm_bf16(M, N, K, ctypes.c_void_p(A.data_ptr()),
                                    ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(C.data_ptr()),
                                    ctypes.c_void_p(err.data_ptr()),
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "fm_tc_gemm_bf16")
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = A.float() @ B.float().T
    scale = (A.float().abs() @ B.float().abs().T)
    assert torch.isfinite(C).all()
    assert ((C - ref).abs() <= 1e-5 * scale + 1e-6).all()
