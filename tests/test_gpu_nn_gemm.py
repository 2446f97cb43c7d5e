"""tcgen05 BF16 GEMM (mflbm_nn_gemm_bf16) against a PyTorch FP32 matmul of the same
bf16 operands.  Both accumulate in FP32; only the summation order differs:
rtol 1e-4, atol 1e-3 for unit-variance inputs."""
import ctypes as C

import pytest

torch = pytest.importorskip("torch")

from mflbm import _capi

pytestmark = pytest.mark.gpu


def _gemm(A, B, Cm=None, accumulate=False):
    lib = _capi.load()
    M, K = A.shape
    N = B.shape[0]
    if Cm is None:
        Cm = torch.zeros(M, N, dtype=torch.float32, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.mflbm_nn_gemm_bf16(A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(0), Cm.data_ptr(), Cm.stride(0),
                                M, N, K, int(accumulate), err.data_ptr(), None)
    assert rc == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return Cm


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (200, 48, 72), (1000, 128, 432), (777, 256, 3456),
                                   (256, 3456, 128), (4096, 32, 896), (130, 64, 8)])
def test_gemm_matches_fp32_reference(M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = _gemm(A, B)
    ref = A.float() @ B.float().t()
    torch.testing.assert_close(C, ref, rtol=1e-4, atol=1e-3)


def test_gemm_accumulates_and_respects_strides():
    g = torch.Generator(device="cuda").manual_seed(5)
    Abig = torch.randn(300, 200, device="cuda", generator=g).to(torch.bfloat16)
    Bbig = torch.randn(64, 136, device="cuda", generator=g).to(torch.bfloat16)
    A = Abig[:, :128]            # lda = 200
    B = Bbig[:48, :128]          # ldb = 136
    C0 = torch.randn(300, 48, device="cuda", generator=g)
    C = _gemm(A, B, C0.clone(), accumulate=True)
    torch.testing.assert_close(C, C0 + A.float() @ B.float().t(), rtol=1e-4, atol=1e-3)


def test_gemm_rejects_bad_shapes():
    lib = _capi.load()
    A = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
    Cm = torch.zeros(128, 24, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    # N = 24 is not a multiple of 16
    assert lib.mflbm_nn_gemm_bf16(A.data_ptr(), 64, A.data_ptr(), 64, Cm.data_ptr(), 24, 128, 24, 64, 0,
                                  err.data_ptr(), None) == _capi.MFLBM_EINVAL
