"""The learned estimator's tcgen05 GEMM (rs_umma.cu: TMA-fed 128-byte-swizzled shared
memory, tcgen05.mma into tensor memory, split over K) against a plain PyTorch FP32 matmul
of the same BF16 operands, and against the mma.sync path, on small and full shapes.

Tolerance: |C - C_ref| <= 1e-5 * (|A| |B|^T) elementwise (FP32 accumulation of the same
BF16 products in another order)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import mlp as omlp
from rayspace3d_gb300 import _lib, learned

pytestmark = pytest.mark.gpu


def _gemm(A, B, mode):
    M, K = A.shape
    N = B.shape[0]
    C = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    st = _lib.load().rs_mlp_gemm(A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(0), C.data_ptr(), C.stride(0), M,
                                 N, K, mode, None)
    return st, C


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (1, 256, 128), (37, 512, 512), (256, 512, 32768), (300, 256, 1024),
                                   (1024, 512, 4096), (4096, 512, 32768)])
def test_umma_gemm_matches_fp32_matmul(cuda, M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    A = (torch.rand(M, K, device="cuda", generator=g) * 4 - 2).to(torch.bfloat16)
    B = (torch.rand(N, K, device="cuda", generator=g) * 4 - 2).to(torch.bfloat16)
    st, C = _gemm(A, B, 0)
    assert st == 0, _lib.status_string(st)
    ref = A.float() @ B.float().T
    bound = 1e-5 * (A.float().abs() @ B.float().abs().T) + 1e-30
    err = (C - ref).abs()
    assert bool(torch.isfinite(C).all())
    assert bool((err <= bound).all()), f"max excess {float((err - bound).max())}"
    st1, C1 = _gemm(A, B, 1)
    assert st1 == 0
    assert bool(((C1 - ref).abs() <= bound).all())


def test_umma_gemm_rejects_shapes_it_cannot_take(cuda):
    A = torch.zeros(4, 96, dtype=torch.bfloat16, device="cuda")
    B = torch.zeros(256, 96, dtype=torch.bfloat16, device="cuda")
    assert _gemm(A, B, 0)[0] == _lib.RS_ERR_INVALID  # K not a multiple of 64
    assert _gemm(A, B, 1)[0] == 0


@pytest.mark.parametrize("B", [1, 24, 256])
def test_forward_paths_agree(cuda, B):
    m = learned.Mlp(seed=5)
    rng = np.random.default_rng(B)
    X = rng.uniform(0.0, 4.0, size=(B, 32768)).astype(np.float32)
    X[:, rng.random(32768) < 0.7] = 0.0
    dX = torch.from_numpy(X).cuda()
    L = _lib.load()
    try:
        L.rs_mlp_set_gemm(0)
        y0 = m.forward(dX).cpu().numpy()
        L.rs_mlp_set_gemm(1)
        y1 = m.forward(dX).cpu().numpy()
    finally:
        L.rs_mlp_set_gemm(0)
    want, _ = omlp.forward(m.params(), X)
    for y in (y0, y1):
        assert np.linalg.norm(y - want) <= 1e-3 * max(np.linalg.norm(want), 1e-30)
    m.close()
