"""GPU parity of the Ozaki (BF16 tcgen05) FP64-emulation path.

Two kinds of checks:
  * bit-exact against the numpy restatement of the same splitting / recombination
    (oracle.ozaki_gemm), which pins the tensor-core pipeline, TMA layouts and epilogue;
  * accuracy against near-exact sampled dot products (Dot2) and the FP64 oracle: the
    normwise error ||C - C_ref||_F / (||A||_F ||B||_F) stays below the returned bound
    and, with automatic slicing, below the native FP64 kernel's error.
"""
import numpy as np
import pytest
import torch

import gbblas
from gbblas import workloads
import oracle
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu


def _run(A, B, C=None, alpha=1.0, beta=0.0, slices=0, ta=0, tb=0, want_bound=False):
    """A, B stored (op via ta/tb); returns (C_host, bound)."""
    M = A.shape[1] if ta else A.shape[0]
    K = A.shape[0] if ta else A.shape[1]
    N = B.shape[0] if tb else B.shape[1]
    Cd = to_dev(C if C is not None else np.zeros((M, N)))
    Ad, Bd = to_dev(A), to_dev(B)
    bound = gbblas.gemm_raw(ta, tb, M, N, K, alpha, Ad.data_ptr(), max(1, A.shape[0]), Bd.data_ptr(),
                            max(1, B.shape[0]), beta, Cd.data_ptr(), max(1, M), dtype=torch.float64,
                            mode=gbblas.MODE_OZAKI_BF16, slices=slices, want_bound=want_bound,
                            stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    return to_host(Cd), bound


SHAPES = [(1, 1, 1), (7, 5, 3), (128, 64, 256), (129, 200, 257), (300, 130, 77), (256, 1000, 384),
          (200, 4100, 130)]


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
@pytest.mark.parametrize("slices", [1, 4, 9])
def test_bit_exact_vs_restatement(cuda, shape, slices):
    M, K, N = shape
    g = np.random.default_rng(M + 3 * K + 7 * N + slices)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-8, 9, (M, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-8, 9, (K, N))))
    got, _ = _run(A, B, slices=slices)
    ref = oracle.ozaki_gemm(A, B, slices=slices)
    assert_bit_equal(got, ref)


@pytest.mark.parametrize("trans", [(0, 1), (1, 0), (1, 1)])
def test_transposes_and_alpha_beta(cuda, trans):
    ta, tb = trans
    M, K, N = 150, 300, 140
    g = np.random.default_rng(17 + ta + 2 * tb)
    Al = g.uniform(-1, 1, (M, K))
    Bl = g.uniform(-1, 1, (K, N))
    C = np.asfortranarray(g.uniform(-1, 1, (M, N)))
    A = np.asfortranarray(Al.T if ta else Al)
    B = np.asfortranarray(Bl.T if tb else Bl)
    got, _ = _run(A, B, C=C, alpha=1.5, beta=0.5, slices=6, ta=ta, tb=tb)
    ref = oracle.ozaki_gemm(Al, Bl, C=C, alpha=1.5, beta=0.5, slices=6)
    assert_bit_equal(got, ref)


@pytest.mark.parametrize("shape", [(300, 8192, 260), (256, 4096, 512), (130, 1000, 70)])
def test_auto_plan_bit_exact(cuda, shape):
    """slices = 0: the library picks slices and K chunking; the result equals the restatement
    of the plan it reports."""
    M, K, N = shape
    A = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=61))
    B = np.asfortranarray(workloads.ozaki_matrix(K, N, per="col", stream=62))
    got, bound = _run(A, B, slices=0, want_bound=True)
    plan = gbblas.last_ozaki_plan()
    assert bound <= 2.0 ** -50
    ref = oracle.ozaki_gemm(A, B, slices=plan["slices"], min_chunks=oracle.chunks_for(K, plan["k_chunk"]))
    assert_bit_equal(got, ref)


def test_chunked_k(cuda):
    """K > 65536 takes two exact accumulation chunks per slice pair."""
    M, K, N = 64, 70000, 40
    g = np.random.default_rng(23)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    got, _ = _run(A, B, slices=3)
    ref = oracle.ozaki_gemm(A, B, slices=3)
    assert_bit_equal(got, ref)


def test_nonfinite_rows_and_columns_give_nan(cuda):
    g = np.random.default_rng(5)
    A = np.asfortranarray(g.uniform(-1, 1, (40, 50)))
    B = np.asfortranarray(g.uniform(-1, 1, (50, 30)))
    A[3, 7] = np.inf
    B[9, 4] = np.nan
    got, _ = _run(A, B, slices=5)
    assert np.isnan(got[3, :]).all() and np.isnan(got[:, 4]).all()
    mask = np.ones_like(got, bool)
    mask[3, :] = False
    mask[:, 4] = False
    assert np.isfinite(got[mask]).all()


def test_beta_zero_ignores_nan_c(cuda):
    g = np.random.default_rng(6)
    A = np.asfortranarray(g.uniform(-1, 1, (33, 44)))
    B = np.asfortranarray(g.uniform(-1, 1, (44, 55)))
    C = np.full((33, 55), np.nan, order="F")
    got, _ = _run(A, B, C=C, slices=4)
    assert np.isfinite(got).all()


def _normwise_err(got, A, B, rows, cols, trans_a=False, trans_b=False):
    hi, lo, _ = oracle.dot2_entries(A, B, rows, cols, trans_a, trans_b)
    d = (got[rows, cols] - hi) - lo
    scale = np.sqrt(got.size / rows.size)   # sampled estimate of the Frobenius norm
    return np.linalg.norm(d) * scale / (np.linalg.norm(A) * np.linalg.norm(B))


@pytest.mark.parametrize("dist", ["uniform", "ozaki"])
def test_accuracy_auto_slices_beats_native(cuda, dist):
    M = K = N = 1024
    if dist == "uniform":
        A = workloads.uniform(M, K, stream=31)
        B = workloads.uniform(K, N, stream=32)
    else:
        A = workloads.ozaki_matrix(M, K, per="row", stream=31)
        B = workloads.ozaki_matrix(K, N, per="col", stream=32)
    oz, bound = _run(A, B, slices=0, want_bound=True)
    Cn = torch.zeros((N, M), dtype=torch.float64, device=cuda).t()
    gbblas.gemm_(Cn, to_dev(A), to_dev(B), mode="native")
    nat = to_host(Cn)
    g = np.random.default_rng(2)
    rows, cols = g.integers(0, M, 4096), g.integers(0, N, 4096)
    e_oz = _normwise_err(oz, A, B, rows, cols)
    e_nat = _normwise_err(nat, A, B, rows, cols)
    assert e_oz <= bound
    assert bound <= 2.0 ** -50 * 1.0001
    assert e_oz <= e_nat, (e_oz, e_nat)


def test_bound_decreases_with_slices_and_holds(cuda):
    M, K, N = 256, 2048, 256
    A = workloads.ozaki_matrix(M, K, per="row", stream=41)
    B = workloads.ozaki_matrix(K, N, per="col", stream=42)
    g = np.random.default_rng(3)
    rows, cols = g.integers(0, M, 2048), g.integers(0, N, 2048)
    prev = np.inf
    for s in (3, 5, 7, 9, 11):
        got, bound = _run(A, B, slices=s, want_bound=True)
        err = _normwise_err(got, A, B, rows, cols)
        assert err <= bound, (s, err, bound)
        assert bound < prev
        prev = bound


def test_int8_mode_unsupported(cuda):
    d = torch.zeros((8, 8), dtype=torch.float64, device=cuda)
    with pytest.raises(gbblas.GBError) as e:
        gbblas.gemm_(d, d, d, mode="ozaki_int8")
    assert e.value.status == gbblas._lib.GB_ERR_UNSUPPORTED


def test_8192_cubed_accuracy_beats_native(cuda):
    """At full size: M = N = K = 8192, sign*U[1,2)*2^(e_line + e_elem) inputs, slices
    chosen by the library; normwise error (4096 Dot2-sampled entries) below the bound and
    below the native FP64 kernel's on the same inputs."""
    n = 8192
    A = np.asfortranarray(workloads.ozaki_matrix(n, n, per="row", stream=1))
    B = np.asfortranarray(workloads.ozaki_matrix(n, n, per="col", stream=2))
    Ad, Bd = to_dev(A), to_dev(B)
    C = torch.empty((n, n), dtype=torch.float64, device=cuda).t()
    _, bound = gbblas.gemm_(C, Ad, Bd, mode="ozaki", return_bound=True)
    oz = to_host(C)
    gbblas.gemm_(C, Ad, Bd, mode="native")
    nat = to_host(C)
    g = np.random.default_rng(12345)
    rows, cols = g.integers(0, n, 4096), g.integers(0, n, 4096)
    e_oz = _normwise_err(oz, A, B, rows, cols)
    e_nat = _normwise_err(nat, A, B, rows, cols)
    assert e_oz <= bound <= 2.0 ** -50
    assert e_oz <= e_nat, (e_oz, e_nat)
