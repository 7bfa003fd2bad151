"""GPU parity of the native FP64/FP32 path (C ABI through ctypes) against the oracle.

The native kernels compute jmul!'s FMA chain in the reference's order, so every check
here is bit-exact (NaN positions compared as positions: payloads are not IEEE-defined).
"""
import glob
import os

import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib
import oracle
from gpu_util import assert_bit_equal, to_dev, to_dev_ld, to_host

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_jmul_matches_golden(cuda, path):
    z = np.load(path)
    A, X, D = z["A"], z["X"], z["D"]
    Dg = torch.full(D.shape, float("nan"), dtype=torch.float64 if D.dtype == np.float64 else torch.float32,
                    device=cuda).t().contiguous().t()
    out = gbblas.jmul_(Dg, to_dev(A), to_dev(X))
    assert out is Dg
    torch.cuda.synchronize()
    assert_bit_equal(to_host(Dg), D)


SHAPES = [(1, 1, 1), (7, 5, 3), (127, 65, 129), (129, 200, 127), (300, 1, 17), (65, 300, 130), (256, 256, 256)]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape", SHAPES, ids=[ "x".join(map(str, s)) for s in SHAPES])
@pytest.mark.parametrize("trans", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_gemm_bit_exact(cuda, dtype, shape, trans):
    M, K, N = shape
    ta, tb = trans
    g = np.random.default_rng(M * 1000 + K * 7 + N + 13 * ta + 29 * tb)
    A = np.asfortranarray(g.uniform(-1, 1, (K, M) if ta else (M, K)).astype(dtype))
    B = np.asfortranarray(g.uniform(-1, 1, (N, K) if tb else (K, N)).astype(dtype))
    C = np.asfortranarray(g.uniform(-1, 1, (M, N)).astype(dtype))
    for alpha, beta in ((1.0, 0.0), (1.5, 0.5), (-2.0, 1.0)):
        ref = oracle.gemm(A, B, C=C, alpha=alpha, beta=beta, trans_a=bool(ta), trans_b=bool(tb), dtype=dtype)
        Cd = to_dev(C)
        Ad, Bd = to_dev(A), to_dev(B)
        gbblas.gemm_raw(ta, tb, M, N, K, alpha, Ad.data_ptr(), max(1, A.shape[0]), Bd.data_ptr(),
                        max(1, B.shape[0]), beta, Cd.data_ptr(), max(1, M),
                        dtype=torch.float64 if dtype == np.float64 else torch.float32,
                        stream=torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert_bit_equal(to_host(Cd), ref)


# Products large enough that FP32 runs its 128 x 128 tile (16-deep K panel) and FP64 its 64 x 64
# tile, with M and N off the tile grid, K ending inside a K panel, and every leading dimension
# padded (NaN in A and B: a load from the padding would poison the result; C's padding must stay).
BIG_TILE_SHAPES = [(1601, 37, 1555), (1700, 129, 1650), (1543, 16, 1675)]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape", BIG_TILE_SHAPES, ids=["x".join(map(str, s)) for s in BIG_TILE_SHAPES])
@pytest.mark.parametrize("trans", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_gemm_large_tiles_ragged_edges(cuda, dtype, shape, trans):
    M, K, N = shape
    ta, tb = trans
    g = np.random.default_rng(M + 3 * K + 7 * N + 11 * ta + 13 * tb)
    A = np.asfortranarray(g.uniform(-1, 1, (K, M) if ta else (M, K)).astype(dtype))
    B = np.asfortranarray(g.uniform(-1, 1, (N, K) if tb else (K, N)).astype(dtype))
    C = np.asfortranarray(g.uniform(-1, 1, (M, N)).astype(dtype))
    ref = oracle.gemm(A, B, C=C, alpha=1.5, beta=0.5, trans_a=bool(ta), trans_b=bool(tb), dtype=dtype)
    lda, ldb, ldc = A.shape[0] + 5, B.shape[0] + 3, M + 2
    Av, _ = to_dev_ld(A, lda)
    Bv, _ = to_dev_ld(B, ldb)
    Cv, Cbuf = to_dev_ld(C, ldc, fill=7.0)
    gbblas.gemm_raw(ta, tb, M, N, K, 1.5, Av.data_ptr(), lda, Bv.data_ptr(), ldb, 0.5, Cv.data_ptr(), ldc,
                    dtype=torch.float64 if dtype == np.float64 else torch.float32,
                    stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert_bit_equal(to_host(Cv), ref)
    assert np.all(to_host(Cbuf)[M:, :] == 7.0), "rows beyond M inside the leading dimension were touched"


def test_jmul_256_cubed_uniform(cuda):
    """Plain Float64 256^3, uniform[-1,1), alpha=1, beta=0: identical to jmul!'s chain."""
    from gbblas import workloads
    A = workloads.uniform(256, 256, stream=1)
    B = workloads.uniform(256, 256, stream=2)
    ref = oracle.jmul(A, B)
    D = torch.empty((256, 256), dtype=torch.float64, device=cuda).t()
    gbblas.jmul_(D, to_dev(A), to_dev(B))
    torch.cuda.synchronize()
    assert_bit_equal(to_host(D), ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_leading_dimensions_larger_than_rows(cuda, dtype):
    g = np.random.default_rng(3)
    M, K, N = 70, 33, 45
    A = g.uniform(-1, 1, (M, K)).astype(dtype)
    B = g.uniform(-1, 1, (K, N)).astype(dtype)
    C = g.uniform(-1, 1, (M, N)).astype(dtype)
    Av, _ = to_dev_ld(A, 80)
    Bv, _ = to_dev_ld(B, 40)
    Cv, Cbuf = to_dev_ld(C, 77, fill=7.0)
    gbblas.gemm_(Cv, Av, Bv, 1.5, 0.5)
    torch.cuda.synchronize()
    ref = oracle.gemm(A, B, C=C, alpha=1.5, beta=0.5, dtype=dtype)
    assert_bit_equal(to_host(Cv), ref)
    full = to_host(Cbuf)
    assert np.all(full[M:, :] == 7.0), "rows beyond M inside the leading dimension were touched"


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_blas_edge_semantics(cuda, dtype):
    A = torch.ones((5, 3), dtype=dtype, device=cuda).t().contiguous().t()
    B = torch.ones((3, 4), dtype=dtype, device=cuda).t().contiguous().t()
    C = torch.full((5, 4), float("nan"), dtype=dtype, device=cuda).t().contiguous().t()
    gbblas.gemm_(C, A, B, 2.0, 0.0)             # beta == 0 overwrites NaN
    assert torch.all(C == 6.0)
    An = torch.full((5, 3), float("nan"), dtype=dtype, device=cuda).t().contiguous().t()
    gbblas.gemm_(C, An, B, 0.0, 0.5)            # alpha == 0: A, B not read
    assert torch.all(C == 3.0)
    A0 = torch.empty((5, 0), dtype=dtype, device=cuda)
    B0 = torch.empty((0, 4), dtype=dtype, device=cuda)
    gbblas.gemm_raw(0, 0, 5, 4, 0, 1.0, A0.data_ptr() or C.data_ptr(), 5, B0.data_ptr() or C.data_ptr(),
                    1, 2.0, C.data_ptr(), 5, dtype=dtype, stream=torch.cuda.current_stream().cuda_stream)
    assert torch.all(C == 6.0)                  # K == 0: C = beta*C
    gbblas.gemm_raw(0, 0, 0, 4, 3, 1.0, 0, 1, 0, 3, 0.0, 0, 1, dtype=dtype,
                    stream=torch.cuda.current_stream().cuda_stream)  # M == 0: no-op


def test_nan_inf_propagation_matches_oracle(cuda):
    g = np.random.default_rng(4)
    A = np.asfortranarray(g.uniform(-1, 1, (40, 30)))
    B = np.asfortranarray(g.uniform(-1, 1, (30, 20)))
    A[3, 5] = np.inf
    A[7, :] = 0.0
    B[5, 0] = 0.0          # inf * 0 -> NaN in C[3, 0]
    A[10, 2] = np.nan
    B[4, 9] = -np.inf
    ref = oracle.jmul(A, B)
    D = torch.empty((20, 40), dtype=torch.float64, device=cuda).t()
    gbblas.jmul_(D, to_dev(A), to_dev(B))
    torch.cuda.synchronize()
    assert_bit_equal(to_host(D), ref)


def test_row_major_tensors(cuda):
    g = np.random.default_rng(11)
    A = g.uniform(-1, 1, (50, 40))
    B = g.uniform(-1, 1, (40, 30))
    C = torch.zeros((50, 30), dtype=torch.float64, device=cuda)        # row-major
    gbblas.gemm_(C, torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda())
    torch.cuda.synchronize()
    # row-major C is computed as C^T = B^T A^T: the per-element chain is the same
    assert_bit_equal(np.asfortranarray(C.cpu().numpy()), oracle.gemm(A, B))


def test_invalid_arguments_return_status(cuda):
    d = torch.zeros((16, 16), dtype=torch.float64, device=cuda)
    p = d.data_ptr()
    s = torch.cuda.current_stream().cuda_stream
    with pytest.raises(gbblas.GBError) as e:
        gbblas.gemm_raw(0, 0, 16, 16, 16, 1.0, p, 8, p, 16, 0.0, p, 16, dtype=torch.float64, stream=s)
    assert e.value.status == _lib.GB_ERR_INVALID_VALUE
    with pytest.raises(gbblas.GBError) as e:
        gbblas.gemm_raw(2, 0, 16, 16, 16, 1.0, p, 16, p, 16, 0.0, p, 16, dtype=torch.float64, stream=s)
    assert e.value.status == _lib.GB_ERR_INVALID_VALUE
    host = np.zeros((16, 16))
    with pytest.raises(gbblas.GBError) as e:
        gbblas.gemm_raw(0, 0, 16, 16, 16, 1.0, host.ctypes.data, 16, p, 16, 0.0, p, 16,
                        dtype=torch.float64, stream=s)
    assert e.value.status == _lib.GB_ERR_INVALID_VALUE
    with pytest.raises(gbblas.GBError) as e:
        gbblas.gemm_raw(0, 0, 16, 16, 16, 1.0, p, 16, p, 16, 0.0, p, 16, dtype=torch.float64,
                        mode=_lib.MODE_OZAKI_INT8, stream=s)
    assert e.value.status == _lib.GB_ERR_UNSUPPORTED
    with pytest.raises(gbblas.DimensionMismatch):
        gbblas.gemm_(d, d[:, :8], d)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gemm_1024_cubed_full_oracle(cuda, dtype):
    """1024^3, alpha=1.5, beta=0.5: every element equals the oracle's."""
    from gbblas import workloads
    n = 1024
    A = workloads.uniform(n, n, stream=11, dtype=dtype)
    B = workloads.uniform(n, n, stream=12, dtype=dtype)
    C = workloads.uniform(n, n, stream=13, dtype=dtype)
    ref = oracle.gemm(A, B, C=C, alpha=1.5, beta=0.5, dtype=dtype)
    Cd = to_dev(C)
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), 1.5, 0.5)
    torch.cuda.synchronize()
    assert_bit_equal(to_host(Cd), ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape", [(2048, 2048, 2048), (4096, 4096, 4096), (16384, 16384, 64),
                                   (64, 16384, 16384)], ids=["2048", "4096", "tall", "wide"])
def test_gemm_large_shapes_sampled_entries(cuda, dtype, shape):
    """Large square and tall/wide shapes (M, K, N): 4096 sampled entries equal the oracle chain."""
    from gbblas import workloads
    M, K, N = shape
    A = workloads.uniform(M, K, stream=21, dtype=dtype)
    B = workloads.uniform(K, N, stream=22, dtype=dtype)
    C = workloads.uniform(M, N, stream=23, dtype=dtype)
    Cd = to_dev(C)
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), 1.5, 0.5)
    g = np.random.default_rng(1)
    rows = g.integers(0, M, 4096)
    cols = g.integers(0, N, 4096)
    ref = oracle.chain_entries(A, B, rows, cols, C=C, alpha=1.5, beta=0.5, dtype=dtype)
    torch.cuda.synchronize()
    got = Cd[torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda()].cpu().numpy()
    assert_bit_equal(got, ref)


def test_native_fp64_error_within_standard_bound_against_binary128(cuda):
    """8192^3 FP64 (alpha = 1, beta = 0): 2048 sampled entries against the binary128 oracle
    lie within the standard bound gamma_K sum |a||b| (gamma_K = K u / (1 - K u), u = 2^-53),
    and the binary128 and Dot2 references agree within Dot2's own error bound."""
    from gbblas import workloads
    M = N = K = 8192
    A = workloads.uniform(M, K, stream=31)
    B = workloads.uniform(K, N, stream=32)
    Cd = torch.empty((N, M), dtype=torch.float64, device=cuda).t()
    gbblas.gemm_(Cd, to_dev(A), to_dev(B))
    g = np.random.default_rng(4)
    rows = g.integers(0, M, 2048)
    cols = g.integers(0, N, 2048)
    qhi, qlo = oracle.quad_entries(A, B, rows, cols)
    dhi, dlo, ab = oracle.dot2_entries(A, B, rows, cols)
    torch.cuda.synchronize()
    got = Cd[torch.from_numpy(rows).cuda(), torch.from_numpy(cols).cuda()].cpu().numpy()
    u = 2.0 ** -53
    gamma = K * u / (1 - K * u)
    err = np.abs((got - qhi) - qlo)
    assert np.all(err <= gamma * ab)
    # Dot2 (Ogita-Rump-Oishi): |error| <= u^2 |x| + gamma_K^2 sum|a||b| for the double-double
    assert np.all(np.abs((dhi - qhi) + (dlo - qlo)) <= 2 * (K * u) ** 2 * ab + 2.0 ** -104 * np.abs(qhi))
