"""Strided batched GEMM (the batch form of jBLAS's fastmul!/kernel!, src/kernels.jl:1-208):
every product bit-identical to the jmul! FMA-chain oracle, FP64 and FP32."""
import numpy as np
import pytest
import torch

import gbblas
import oracle
from gpu_util import assert_bit_equal

pytestmark = pytest.mark.gpu


def _dev_batch(X):
    """numpy (count, r, c) -> CUDA (count, r, c) with column-major matrices."""
    return torch.from_numpy(np.ascontiguousarray(np.transpose(X, (0, 2, 1)))).cuda().transpose(1, 2)


def _host_batch(T):
    return np.ascontiguousarray(T.detach().cpu().numpy())


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape", [(7, 5, 3), (33, 17, 65), (128, 96, 40), (1, 1, 1), (200, 3, 150)])
def test_strided_batched_bit_exact(cuda, dtype, shape):
    M, N, K = shape
    count = 37
    g = np.random.default_rng(M * 7 + N * 3 + K)
    A = g.uniform(-1, 1, (count, M, K)).astype(dtype)
    B = g.uniform(-1, 1, (count, K, N)).astype(dtype)
    C = g.uniform(-1, 1, (count, M, N)).astype(dtype)
    Cd = _dev_batch(C)
    gbblas.gemm_strided_batched_(Cd, _dev_batch(A), _dev_batch(B), 1.5, 0.5)
    torch.cuda.synchronize()
    got = _host_batch(Cd)
    for i in (0, count // 2, count - 1):
        ref = oracle.gemm(A[i], B[i], C=C[i], alpha=1.5, beta=0.5, dtype=dtype)
        assert_bit_equal(np.asfortranarray(got[i]), ref)


def test_broadcast_operand_and_beta_zero(cuda):
    M, N, K, count = 24, 40, 56, 64
    g = np.random.default_rng(4)
    A = g.uniform(-1, 1, (M, K))
    B = g.uniform(-1, 1, (count, K, N))
    Ad = _dev_batch(A[None]).expand(count, M, K)   # stride 0 along the batch
    Cd = torch.full((count, N, M), float("nan"), dtype=torch.float64, device=cuda).transpose(1, 2)
    gbblas.gemm_strided_batched_(Cd, Ad, _dev_batch(B))
    got = _host_batch(Cd)
    for i in (0, 17, count - 1):
        assert_bit_equal(np.asfortranarray(got[i]), oracle.gemm(A, B[i]))


def test_overlapping_outputs_rejected(cuda):
    A = torch.zeros((4, 8, 8), dtype=torch.float64, device=cuda)
    B = torch.zeros((4, 8, 8), dtype=torch.float64, device=cuda)
    C = torch.zeros((8, 8), dtype=torch.float64, device=cuda).t()[None].expand(4, 8, 8)   # one C for all
    with pytest.raises(gbblas.GBError) as e:
        gbblas.gemm_strided_batched_(C, A.transpose(1, 2), B.transpose(1, 2))
    assert e.value.status == gbblas._lib.GB_ERR_INVALID_VALUE
