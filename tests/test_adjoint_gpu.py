"""GPU checks of the fused adjoint (dA = dC B^T, dB = A^T dC, 3xBF16 split, FP32 accumulation).

Stated tolerance (componentwise): the 3xBF16 split drops the lo*lo term and rounds hi and
lo to BF16, so each product carries a relative error below 2^-15; FP32 accumulation over
the contraction length L adds at most L * 2^-24 relative to the sum of |terms|:
    |dA - dA_ref|_ik <= (2^-15 + L * 2^-24) * (|dC| |B|^T)_ik
Checks are against the FP64 oracle on transposed operands (jmul!'s chain on dC and B^T)
and, at the full 4096 x 2048 x 4096 shape, against Float64 central finite differences.
"""
import numpy as np
import pytest
import torch

import gbblas
from gbblas import workloads
import oracle
from gpu_util import to_dev, to_host

pytestmark = pytest.mark.gpu


def tol_factor(L):
    return 2.0 ** -15 + L * 2.0 ** -24


def run_adjoint(A, B, W):
    M, K = A.shape
    N = B.shape[1]
    dA = torch.full((K, M), float("nan"), dtype=torch.float32, device="cuda").t()
    dB = torch.full((N, K), float("nan"), dtype=torch.float32, device="cuda").t()
    gbblas.gemm_adjoint_(dA, dB, to_dev(A), to_dev(B), to_dev(W))
    torch.cuda.synchronize()
    gbblas.check_device_status()
    return to_host(dA), to_host(dB)


SHAPES = [(1, 1, 1), (7, 5, 3), (130, 260, 70), (257, 129, 300), (64, 64, 64), (300, 513, 129)]


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
def test_matches_oracle_on_transposed_operands(cuda, shape):
    M, N, K = shape
    g = np.random.default_rng(M + 7 * N + 13 * K)
    A = np.asfortranarray(g.standard_normal((M, K)).astype(np.float32))
    B = np.asfortranarray(g.standard_normal((K, N)).astype(np.float32))
    W = np.asfortranarray(g.standard_normal((M, N)).astype(np.float32))
    dA, dB = run_adjoint(A, B, W)
    A64, B64, W64 = A.astype(np.float64), B.astype(np.float64), W.astype(np.float64)
    dA_ref = oracle.gemm(W64, B64, trans_b=True)          # dC * B^T
    dB_ref = oracle.gemm(A64, W64, trans_a=True)          # A^T * dC
    absA = np.abs(W64) @ np.abs(B64).T
    absB = np.abs(A64).T @ np.abs(W64)
    assert np.all(np.abs(dA - dA_ref) <= tol_factor(N) * absA + 1e-30)
    assert np.all(np.abs(dB - dB_ref) <= tol_factor(M) * absB + 1e-30)


def test_empty_contraction_gives_zero_gradients(cuda):
    A = np.zeros((5, 3), np.float32, order="F")
    B = np.zeros((3, 0), np.float32, order="F")
    W = np.zeros((5, 0), np.float32, order="F")
    dA = torch.full((3, 5), float("nan"), dtype=torch.float32, device="cuda").t()
    dB = torch.empty((0, 3), dtype=torch.float32, device="cuda").t()
    gbblas.gemm_adjoint_(dA, dB, to_dev(A), to_dev(B), to_dev(W))
    torch.cuda.synchronize()
    assert torch.all(dA == 0)


def test_autograd_function_uses_the_adjoint(cuda):
    g = np.random.default_rng(3)
    A = to_dev(g.standard_normal((96, 80)).astype(np.float32)).requires_grad_(True)
    B = to_dev(g.standard_normal((80, 72)).astype(np.float32)).requires_grad_(True)
    W = to_dev(g.standard_normal((96, 72)).astype(np.float32))
    C = gbblas.gemm_autograd(A, B)
    (C * W).sum().backward()
    dA = torch.empty((80, 96), dtype=torch.float32, device="cuda").t()
    dB = torch.empty((72, 80), dtype=torch.float32, device="cuda").t()
    gbblas.gemm_adjoint_(dA, dB, A.detach(), B.detach(), W)
    assert torch.equal(A.grad, dA) and torch.equal(B.grad, dB)
    # forward is the native FP32 jmul! chain
    ref = oracle.gemm(to_host(A.detach()), to_host(B.detach()), dtype=np.float32)
    assert np.array_equal(to_host(C.detach()), ref)


def test_adjoint_4096x2048x4096_fd_and_oracle(cuda):
    """loss = sum(W .* (A*B)), A 4096x2048, B 2048x4096, W 4096x4096, N(0,1) float32."""
    M, K, N = 4096, 2048, 4096
    A = np.asfortranarray(workloads.normal(M, K, stream=51))
    B = np.asfortranarray(workloads.normal(K, N, stream=52))
    W = np.asfortranarray(workloads.normal(M, N, stream=53))
    dA, dB = run_adjoint(A, B, W)
    A64, B64, W64 = (np.asarray(x, dtype=np.float64) for x in (A, B, W))
    g = np.random.default_rng(4)
    h = 1e-6
    # Float64 central differences of the loss on 64 entries of A and 64 of B.  The loss
    # change from perturbing A[i,k] is confined to row i of A*B, so the two loss values are
    # evaluated on that row only (the other rows cancel exactly).
    for _ in range(64):
        i, k = int(g.integers(M)), int(g.integers(K))
        r = B64 @ W64[i, :]                       # d loss / d A[i, :] direction
        a = A64[i, :].copy()
        ap, am = a.copy(), a.copy()
        ap[k] += h
        am[k] -= h
        fd = (ap @ r - am @ r) / (2 * h)
        scale = np.abs(W64[i, :]) @ np.abs(B64[k, :])
        assert abs(dA[i, k] - fd) <= tol_factor(N) * scale + 1e-6 * abs(fd) + 1e-9, (i, k, dA[i, k], fd)
    for _ in range(64):
        k, j = int(g.integers(K)), int(g.integers(N))
        r = A64.T @ W64[:, j]
        b = B64[:, j].copy()
        bp, bm = b.copy(), b.copy()
        bp[k] += h
        bm[k] -= h
        fd = (r @ bp - r @ bm) / (2 * h)
        scale = np.abs(A64[:, k]) @ np.abs(W64[:, j])
        assert abs(dB[k, j] - fd) <= tol_factor(M) * scale + 1e-6 * abs(fd) + 1e-9, (k, j, dB[k, j], fd)
    # against the reference chain on transposed operands (FP64, 4096 sampled entries each)
    rows, cols = g.integers(0, M, 4096), g.integers(0, K, 4096)
    ref = oracle.chain_entries(W64, B64, rows, cols, trans_b=True)
    _, _, absd = oracle.dot2_entries(np.abs(W64), np.abs(B64), rows, cols, trans_b=True)
    assert np.all(np.abs(dA[rows, cols] - ref) <= tol_factor(N) * absd)
    rows, cols = g.integers(0, K, 4096), g.integers(0, N, 4096)
    ref = oracle.chain_entries(A64, W64, rows, cols, trans_a=True)
    _, _, absd = oracle.dot2_entries(np.abs(A64), np.abs(W64), rows, cols, trans_a=True)
    assert np.all(np.abs(dB[rows, cols] - ref) <= tol_factor(M) * absd)
    # normwise, for the record: well inside 2^-15
    e = np.linalg.norm(dA[rows % M, cols % K] - oracle.chain_entries(W64, B64, rows % M, cols % K, trans_b=True))
    assert e / np.linalg.norm(oracle.chain_entries(W64, B64, rows % M, cols % K, trans_b=True)) < 2.0 ** -14


def test_leading_dimensions_larger_than_rows(cuda):
    """A, B, dC inside larger column-major buffers and dA, dB written into padded ones: the same
    tolerance as packed operands, and the gradients' padding rows are not written."""
    from gpu_util import to_dev_ld
    M, N, K = 150, 97, 133
    g = np.random.default_rng(808)
    A = np.asfortranarray(g.standard_normal((M, K)).astype(np.float32))
    B = np.asfortranarray(g.standard_normal((K, N)).astype(np.float32))
    W = np.asfortranarray(g.standard_normal((M, N)).astype(np.float32))
    Ad, _ = to_dev_ld(A, M + 11)
    Bd, _ = to_dev_ld(B, K + 5)
    Wd, _ = to_dev_ld(W, M + 3)
    dAd, dAbuf = to_dev_ld(np.zeros((M, K), np.float32), M + 9, fill=7.0)
    dBd, dBbuf = to_dev_ld(np.zeros((K, N), np.float32), K + 2, fill=7.0)
    gbblas.gemm_adjoint_(dAd, dBd, Ad, Bd, Wd)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    A64, B64, W64 = A.astype(np.float64), B.astype(np.float64), W.astype(np.float64)
    dA_ref = oracle.gemm(W64, B64, trans_b=True)
    dB_ref = oracle.gemm(A64, W64, trans_a=True)
    assert np.all(np.abs(to_host(dAd) - dA_ref) <= tol_factor(N) * (np.abs(W64) @ np.abs(B64).T) + 1e-30)
    assert np.all(np.abs(to_host(dBd) - dB_ref) <= tol_factor(M) * (np.abs(A64).T @ np.abs(W64)) + 1e-30)
    assert np.all(to_host(dAbuf)[M:, :] == 7.0) and np.all(to_host(dBbuf)[K:, :] == 7.0)
