"""FP32 GEMM on the tensor cores (gb_gemm_f32_ex, modes BF16X3 and BF16X6).

Stated tolerance, per element, against the FP64 oracle of the same inputs
(C_ref = alpha op(A) op(B) + beta C0 in FP64, jmul!'s chain on float64 copies):
    |C - C_ref|_ij <= tol(K) |alpha| (|op(A)| |op(B)|)_ij + 2^-23 (|alpha| |op(A) op(B)| + |beta| |C0|)_ij
    tol(K) = 2^-15 + K 2^-24 (BF16X3: two BF16 terms per value, three term products)
    tol(K) = 2^-21 + K 2^-24 (BF16X6: three terms, six products)
The last term covers the FP32 rounding of alpha * sum + beta * C0 in the epilogue.
"""
import ctypes

import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib
import oracle
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu

TOL = {"bf16x3": 2.0 ** -15, "bf16x6": 2.0 ** -21}


def _check(got, A64, B64, C0, alpha, beta, mode, ta=False, tb=False):
    K = A64.shape[0] if ta else A64.shape[1]
    prod = oracle.gemm(A64, B64, trans_a=ta, trans_b=tb)
    absprod = oracle.gemm(np.abs(A64), np.abs(B64), trans_a=ta, trans_b=tb)
    ref = alpha * prod + (beta * C0 if beta != 0 else 0.0)
    bound = (TOL[mode] + K * 2.0 ** -24) * abs(alpha) * absprod + \
        2.0 ** -23 * (abs(alpha) * np.abs(prod) + abs(beta) * np.abs(C0)) + 1e-37
    err = np.abs(got.astype(np.float64) - ref)
    assert np.all(err <= bound), (mode, float(np.max(err / bound)))


SHAPES = [(1, 1, 1), (7, 5, 3), (129, 200, 257), (300, 130, 77), (256, 1000, 384), (513, 4100, 130)]


@pytest.mark.parametrize("mode", ["bf16x3", "bf16x6"])
@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
def test_within_stated_tolerance(cuda, mode, shape):
    M, K, N = shape
    g = np.random.default_rng(M + 3 * K + 5 * N + len(mode))
    A = np.asfortranarray(g.standard_normal((M, K)).astype(np.float32))
    B = np.asfortranarray(g.standard_normal((K, N)).astype(np.float32))
    C0 = np.asfortranarray(g.standard_normal((M, N)).astype(np.float32))
    Cd = to_dev(C0)
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), 1.5, -0.5, mode=mode)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    _check(to_host(Cd), A.astype(np.float64), B.astype(np.float64), C0.astype(np.float64), 1.5, -0.5, mode)


@pytest.mark.parametrize("mode", ["bf16x3", "bf16x6"])
@pytest.mark.parametrize("trans", [(0, 1), (1, 0), (1, 1)])
def test_transposes(cuda, mode, trans):
    ta, tb = trans
    M, K, N = 150, 300, 140
    g = np.random.default_rng(31 + ta + 2 * tb)
    A = np.asfortranarray(g.uniform(-1, 1, (K, M) if ta else (M, K)).astype(np.float32))
    B = np.asfortranarray(g.uniform(-1, 1, (N, K) if tb else (K, N)).astype(np.float32))
    Cd = to_dev(np.zeros((M, N), np.float32))
    Ad, Bd = to_dev(A), to_dev(B)
    gbblas.gemm_raw(ta, tb, M, N, K, 1.0, Ad.data_ptr(), A.shape[0], Bd.data_ptr(), B.shape[0], 0.0,
                    Cd.data_ptr(), M, dtype=torch.float32, mode=_lib.MODE_BF16X3 if mode == "bf16x3" else
                    _lib.MODE_BF16X6, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    _check(to_host(Cd), A.astype(np.float64), B.astype(np.float64), np.zeros((M, N)), 1.0, 0.0, mode, bool(ta),
           bool(tb))


@pytest.mark.parametrize("mode", ["bf16x3", "bf16x6"])
def test_8192_cubed_sampled(cuda, mode):
    """M = N = K = 8192, N(0,1) inputs drawn on the device: a 64 x 64 grid of outputs within the
    stated tolerance of Dot2 references; BF16X6 within 2^-21 + K 2^-24 means FP32-level error."""
    n = 8192
    gen = torch.Generator(device=cuda).manual_seed(2024 + len(mode))
    A = torch.randn((n, n), generator=gen, dtype=torch.float32, device=cuda).t()
    B = torch.randn((n, n), generator=gen, dtype=torch.float32, device=cuda).t()
    C = torch.empty((n, n), dtype=torch.float32, device=cuda).t()
    gbblas.gemm_(C, A, B, mode=mode)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    g = np.random.default_rng(9)
    r = np.sort(g.choice(n, 64, replace=False))
    c = np.sort(g.choice(n, 64, replace=False))
    rt, ct = torch.as_tensor(r, device=cuda), torch.as_tensor(c, device=cuda)
    As = np.asfortranarray(A[rt].double().cpu().numpy())
    Bs = np.asfortranarray(B[:, ct].double().cpu().numpy())
    got = C[rt][:, ct].double().cpu().numpy()
    ii, jj = (x.ravel() for x in np.meshgrid(np.arange(64), np.arange(64), indexing="ij"))
    hi, lo, ab = oracle.dot2_entries(As, Bs, ii, jj)
    err = np.abs((got[ii, jj] - hi) - lo)
    bound = (TOL[mode] + n * 2.0 ** -24) * ab + 2.0 ** -23 * np.abs(hi)
    assert np.all(err <= bound), float(np.max(err / bound))


def test_no_product_cases_equal_native(cuda):
    """alpha = 0 or K = 0: C = beta C, the same bits as the native mode (A and B not read)."""
    g = np.random.default_rng(4)
    C0 = np.asfortranarray(g.uniform(-1, 1, (33, 21)).astype(np.float32))
    A = to_dev(np.ones((33, 5), np.float32))
    B = to_dev(np.ones((5, 21), np.float32))
    for mode in ("bf16x3", "bf16x6"):
        c1, c2 = to_dev(C0), to_dev(C0)
        gbblas.gemm_(c1, A, B, 0.0, 0.75, mode=mode)
        gbblas.gemm_(c2, A, B, 0.0, 0.75)
        torch.cuda.synchronize()
        assert_bit_equal(to_host(c1), to_host(c2))


def test_invalid_mode_rejected(cuda):
    d = torch.zeros((8, 8), dtype=torch.float32, device=cuda)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = ctypes.c_void_p(d.data_ptr())
    for mode in (_lib.MODE_OZAKI_BF16, _lib.MODE_OZAKI_CRT, 6, -1):
        rc = _lib.lib().gb_gemm_f32_ex(0, 0, 8, 8, 8, 1.0, p, 8, p, 8, 0.0, p, 8, mode, st)
        assert rc == _lib.GB_ERR_INVALID_VALUE


@pytest.mark.parametrize("engine", [1, 2], ids=["single_cta", "cta_pair"])
def test_both_engines(cuda, engine):
    M, K, N = 300, 513, 257
    g = np.random.default_rng(77)
    A = np.asfortranarray(g.standard_normal((M, K)).astype(np.float32))
    B = np.asfortranarray(g.standard_normal((K, N)).astype(np.float32))
    gbblas.set_tc_engine(engine)
    try:
        for mode in ("bf16x3", "bf16x6"):
            Cd = to_dev(np.zeros((M, N), np.float32))
            gbblas.gemm_(Cd, to_dev(A), to_dev(B), mode=mode)
            torch.cuda.synchronize()
            gbblas.check_device_status()
            _check(to_host(Cd), A.astype(np.float64), B.astype(np.float64), np.zeros((M, N)), 1.0, 0.0, mode)
    finally:
        gbblas.set_tc_engine(0)
