"""tcgen05 BF16 GEMM (tensor cores, TMEM accumulator) against an FP32
matmul of the same BF16 operands."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _gemm(gpu, A, B, strides=None):
    from photic_gb300 import _lib as L
    M, K = A.shape
    N = B.shape[0]
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    if strides is None:
        rc = L.lib().photic_gemm_bf16(A.data_ptr(), K, B.data_ptr(), K, C.data_ptr(), N, M, N,
                                      K, s)
    else:
        rc = L.lib().photic_gemm_bf16_strides(A.data_ptr(), K, B.data_ptr(), K, C.data_ptr(), N,
                                              M, N, K, strides[0], strides[1], s)
    L.check(rc)
    gpu.sync()
    return C


@pytest.mark.parametrize("M,N,K", [(128, 128, 16), (256, 128, 192), (300, 16, 128),
                                   (1000, 5, 128), (129, 128, 16), (8192, 128, 128)])
def test_gemm_matches_fp32_matmul(gpu, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = _gemm(gpu, A, B)
    ref = A.float() @ B.float().T
    err = (C - ref).abs().max().item()
    assert err <= 1e-3 * max(1.0, ref.abs().max().item()), err
