"""Both tensor-core engines selectable through gb_set_tc_engine give the same results.

Engine 1 runs one CTA per 128 x 256 tile (tcgen05 cta_group::1), engine 2 a CTA pair per
256 x 256 tile (cta_group::2); 0 picks the pair engine.  The digit-slice mode is bit-exact
against its restatement under each engine (its FP32 sums are exact integers, so the engine
cannot change them), and the adjoint stays within its stated componentwise tolerance under
each.  The CRT mode always runs on CTA pairs.
"""
import numpy as np
import pytest
import torch

import gbblas
import oracle
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture(params=[1, 2], ids=["single_cta", "cta_pair"])
def engine(request, cuda):
    gbblas.set_tc_engine(request.param)
    try:
        yield request.param
    finally:
        gbblas.set_tc_engine(0)


SHAPES = [(7, 5, 3), (129, 200, 257), (300, 130, 77), (256, 1000, 384), (513, 4100, 130)]


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
@pytest.mark.parametrize("slices", [3, 9])
def test_slice_mode_bit_exact_under_each_engine(engine, shape, slices):
    M, K, N = shape
    g = np.random.default_rng(M + 5 * K + 11 * N + slices)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-8, 9, (M, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-8, 9, (K, N))))
    C0 = np.asfortranarray(g.uniform(-1, 1, (M, N)))
    Cd = to_dev(C0)
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), 1.25, -0.5, mode="ozaki", slices=slices)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    ref = oracle.ozaki_gemm(A, B, C=C0, alpha=1.25, beta=-0.5, slices=slices)
    assert_bit_equal(to_host(Cd), ref)


def test_slice_mode_multi_chunk_under_each_engine(engine):
    """K cut into four exact accumulation chunks (wider digits, several TMEM drains per tile)."""
    M, K, N = 300, 2048, 260
    g = np.random.default_rng(99)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    gbblas.set_ozaki_min_chunks(4)
    try:
        Cd = to_dev(np.zeros((M, N)))
        gbblas.gemm_(Cd, to_dev(A), to_dev(B), mode="ozaki", slices=6)
        torch.cuda.synchronize()
        gbblas.check_device_status()
    finally:
        gbblas.set_ozaki_min_chunks(0)
    assert_bit_equal(to_host(Cd), oracle.ozaki_gemm(A, B, slices=6, min_chunks=4))


@pytest.mark.parametrize("shape", [(130, 260, 70), (300, 513, 129), (512, 384, 640)],
                         ids=["130x260x70", "300x513x129", "512x384x640"])
def test_adjoint_within_tolerance_under_each_engine(engine, shape):
    M, N, K = shape
    g = np.random.default_rng(M + 3 * N + 5 * K)
    A = np.asfortranarray(g.standard_normal((M, K)).astype(np.float32))
    B = np.asfortranarray(g.standard_normal((K, N)).astype(np.float32))
    W = np.asfortranarray(g.standard_normal((M, N)).astype(np.float32))
    dA = torch.full((K, M), float("nan"), dtype=torch.float32, device="cuda").t()
    dB = torch.full((N, K), float("nan"), dtype=torch.float32, device="cuda").t()
    gbblas.gemm_adjoint_(dA, dB, to_dev(A), to_dev(B), to_dev(W))
    torch.cuda.synchronize()
    gbblas.check_device_status()
    A64, B64, W64 = A.astype(np.float64), B.astype(np.float64), W.astype(np.float64)
    tol = lambda L: 2.0 ** -15 + L * 2.0 ** -24   # noqa: E731
    assert np.all(np.abs(to_host(dA) - oracle.gemm(W64, B64, trans_b=True))
                  <= tol(N) * (np.abs(W64) @ np.abs(B64).T) + 1e-30)
    assert np.all(np.abs(to_host(dB) - oracle.gemm(A64, W64, trans_a=True))
                  <= tol(M) * (np.abs(A64).T @ np.abs(W64)) + 1e-30)
