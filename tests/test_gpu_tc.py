"""tcgen05 BF16 GEMM building block vs a float64 matmul of the same bf16 inputs."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 192), (384, 128, 512)])
def test_tc_gemm_bf16(M, N, K):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from trot_gb300 import _lib, native

    g = torch.Generator().manual_seed(M + N + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    D = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    _lib.call("trot_tc_gemm_bf16", A.data_ptr(), B.data_ptr(), D.data_ptr(), M, N, K, status.data_ptr(),
              native.stream_ptr())
    assert int(status.item()) == 0
    ref = A.double() @ B.double().T
    err = (D.double() - ref).abs().max().item()
    # exact products, fp32 accumulation over K terms
    assert err <= 1e-5 * K ** 0.5 * ref.abs().max().item(), err
