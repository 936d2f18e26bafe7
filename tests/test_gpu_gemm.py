"""K1: the batched max-plus GEMM against a torch fp32 reference."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def maxplus_ref(A, B):
    # A (b, K, M) col-major view -> C (b, N, M)
    return (A.unsqueeze(1) + B.unsqueeze(3)).amax(dim=2)


@pytest.mark.parametrize("shape", [(16, 16, 16, 1), (128, 128, 64, 2), (64, 256, 32, 3), (256, 32, 128, 1),
                                   (32, 128, 16, 4), (512, 512, 256, 1)])
def test_k1_matches_reference(engine, shape):
    import torch

    M, N, K, b = shape
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randint(-50, 50, (b, K, M), device="cuda", generator=g).float()
    B = torch.randint(-50, 50, (b, N, K), device="cuda", generator=g).float()
    A[torch.rand(A.shape, device="cuda", generator=g) < 0.05] = float("-inf")
    C = torch.empty((b, N, M), device="cuda")
    torch.cuda.synchronize()
    engine.gemm(M, N, K, b, A.data_ptr(), B.data_ptr(), C.data_ptr(), None)
    torch.cuda.synchronize()
    ref = torch.stack([maxplus_ref(A[i:i + 1], B[i:i + 1])[0] for i in range(b)])
    assert torch.equal(C, ref)
