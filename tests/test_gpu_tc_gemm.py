"""The tcgen05 BF16 GEMM (C = A B^T, K-major operands, FP32 accumulation in
tensor memory) against an FP64 product of the same BF16-rounded operands,
through the C ABI.  Shapes cover the learned guess's layers, K tails that
are not a multiple of the 64-wide slice, and M, N past one tile.  Bar: 1e-5
relative (FP32 accumulation of up to 2560 products)."""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(300, 64, 2560), (128, 512, 64), (1000, 200, 130), (77, 64, 64),
                                   (64, 512, 3000), (2560, 64, 520)])
def test_gemm_bf16_matches_fp64_product(pkg, dev, M, N, K):
    L = pkg.lib()
    rng = np.random.default_rng(M * 7 + N + K)
    lda = (K + 7) // 8 * 8
    A = rng.standard_normal((M, K)).astype(np.float32)
    B = rng.standard_normal((N, K)).astype(np.float32)
    Ab = np.zeros((M, lda), dtype=np.uint16)
    Bb = np.zeros((N, lda), dtype=np.uint16)
    Ab[:, :K] = mlp_ref.bf16_bits(A)
    Bb[:, :K] = mlp_ref.bf16_bits(B)
    Ad = torch.from_numpy(Ab.view(np.int16)).to(dev)
    Bd = torch.from_numpy(Bb.view(np.int16)).to(dev)
    Cd = torch.full((M, N), float("nan"), dtype=torch.float32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    st = L.ntg_gemm_bf16(C.c_void_p(Ad.data_ptr()), lda, C.c_void_p(Bd.data_ptr()), lda, C.c_void_p(Cd.data_ptr()), N,
                         M, N, K, C.c_void_p(err.data_ptr()), None)
    assert st == 0, L.ntg_last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = mlp_ref.bf16(A).astype(np.float64) @ mlp_ref.bf16(B).astype(np.float64).T
    got = Cd.cpu().numpy().astype(np.float64)
    assert np.isfinite(got).all()
    e = np.abs(got - ref).max() / np.abs(ref).max()
    assert e < 1e-5, e


def test_gemm_bf16_rejects_unaligned_rows(pkg, dev):
    L = pkg.lib()
    A = torch.zeros(64 * 10, dtype=torch.int16, device=dev)
    Cd = torch.zeros(64 * 64, dtype=torch.float32, device=dev)
    st = L.ntg_gemm_bf16(C.c_void_p(A.data_ptr()), 10, C.c_void_p(A.data_ptr()), 10, C.c_void_p(Cd.data_ptr()), 64, 64,
                         64, 10, None, None)
    assert st == 1 and b"aligned" in L.ntg_last_error()
