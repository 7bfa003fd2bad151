"""GPU parity of the CRT (Ozaki scheme II) FP64-emulation mode.

The restatement (oracle.ozaki_crt_gemm) forms the integer product of the t-bit scaled
operands exactly, by a different route than the GPU (limb products instead of residues and
the Chinese remainder theorem), so bit equality pins the residue split, the modular
tensor-core products, the per-chunk reductions, the 128-bit reconstruction and the FP64
rounding together.  Accuracy checks against Dot2-sampled entries as for the slice mode.
"""
import numpy as np
import pytest
import torch

import gbblas
from gbblas import workloads
import oracle
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu


def _run(A, B, C=None, alpha=1.0, beta=0.0, moduli=0, ta=0, tb=0, want_bound=False):
    M = A.shape[1] if ta else A.shape[0]
    K = A.shape[0] if ta else A.shape[1]
    N = B.shape[0] if tb else B.shape[1]
    Cd = to_dev(C if C is not None else np.zeros((M, N)))
    Ad, Bd = to_dev(A), to_dev(B)
    bound = gbblas.gemm_raw(ta, tb, M, N, K, alpha, Ad.data_ptr(), max(1, A.shape[0]), Bd.data_ptr(),
                            max(1, B.shape[0]), beta, Cd.data_ptr(), max(1, M), dtype=torch.float64,
                            mode=gbblas.MODE_OZAKI_CRT, slices=moduli, want_bound=want_bound,
                            stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    return to_host(Cd), bound


SHAPES = [(1, 1, 1), (7, 5, 3), (128, 64, 256), (129, 200, 257), (300, 130, 77), (256, 1000, 384),
          (200, 4100, 130), (513, 96, 260)]


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
@pytest.mark.parametrize("moduli", [3, 8, 16, 20])
def test_bit_exact_vs_restatement(cuda, shape, moduli):
    M, K, N = shape
    g = np.random.default_rng(M + 3 * K + 7 * N + moduli)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-8, 9, (M, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-8, 9, (K, N))))
    got, _ = _run(A, B, moduli=moduli)
    assert gbblas.last_ozaki_plan()["bits"] == oracle.crt_bits_for(K, moduli)
    ref = oracle.ozaki_crt_gemm(A, B, moduli=moduli)
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
    got, _ = _run(A, B, C=C, alpha=1.5, beta=0.5, moduli=14, ta=ta, tb=tb)
    ref = oracle.ozaki_crt_gemm(Al, Bl, C=C, alpha=1.5, beta=0.5, moduli=14)
    assert_bit_equal(got, ref)


def test_extreme_exponents_and_subnormal_results(cuda):
    """Rows and columns scaled near the ends of the FP64 range: results overflow to Inf,
    land in the subnormal range (rounded once from the exact product's FP64 value), or stay
    normal, exactly as the restatement says."""
    M, K, N = 64, 96, 48
    g = np.random.default_rng(77)
    A = g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-4, 5, (M, K)))
    B = g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-4, 5, (K, N)))
    A[:16] *= 2.0 ** 600
    B[:, :12] *= 2.0 ** 600          # A rows 0-15 x B cols 0-11 overflow
    A[16:32] *= 2.0 ** -540
    B[:, 12:24] *= 2.0 ** -520       # subnormal and underflowing products
    A[32:40] *= 2.0 ** -1030         # subnormal inputs
    A, B = np.asfortranarray(A), np.asfortranarray(B)
    got, _ = _run(A, B, moduli=16)
    ref = oracle.ozaki_crt_gemm(A, B, moduli=16)
    assert np.isinf(ref[:16, :12]).any()
    sub = (ref != 0) & (np.abs(ref) < 2.2250738585072014e-308)
    assert sub.any()
    assert_bit_equal(got, ref)


@pytest.mark.parametrize("shape", [(300, 8192, 260), (256, 4096, 512), (130, 1000, 70)])
def test_auto_plan_bit_exact(cuda, shape):
    """moduli = 0: the library picks moduli and t from the operands' statistics; the result
    equals the restatement of the plan it reports, within the tolerance."""
    M, K, N = shape
    A = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=61))
    B = np.asfortranarray(workloads.ozaki_matrix(K, N, per="col", stream=62))
    got, bound = _run(A, B, moduli=0, want_bound=True)
    plan = gbblas.last_ozaki_plan()
    assert bound <= 2.0 ** -50
    ref = oracle.ozaki_crt_gemm(A, B, moduli=plan["slices"], bits=plan["bits"])
    assert_bit_equal(got, ref)


def test_auto_plan_with_subnormal_rows(cuda):
    """Rows whose every entry is subnormal (and columns scaled near the top of the range):
    the statistics scale subnormals exactly, so the automatic t keeps |C'| inside the CRT
    range and the result equals the restatement of the reported plan."""
    M, K, N = 96, 700, 80
    g = np.random.default_rng(91)
    A = g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-3, 4, (M, K)))
    B = g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-3, 4, (K, N)))
    A[:24] *= 2.0 ** -1060      # every entry subnormal
    A[24:30] *= 2.0 ** -1030    # mixed subnormal / normal magnitudes
    B[:, :10] *= 2.0 ** 900
    A, B = np.asfortranarray(A), np.asfortranarray(B)
    got, bound = _run(A, B, moduli=0, want_bound=True)
    plan = gbblas.last_ozaki_plan()
    ref = oracle.ozaki_crt_gemm(A, B, moduli=plan["slices"], bits=plan["bits"])
    assert_bit_equal(got, ref)
    assert bound <= 2.0 ** -50


def test_long_k_many_chunks(cuda):
    """K = 70000: 69 exact accumulation chunks per modulus, summed mod p in the residue planes."""
    M, K, N = 64, 70000, 40
    g = np.random.default_rng(23)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    got, _ = _run(A, B, moduli=18)
    ref = oracle.ozaki_crt_gemm(A, B, moduli=18)
    assert_bit_equal(got, ref)


def test_nonfinite_rows_and_columns_give_nan(cuda):
    g = np.random.default_rng(5)
    A = np.asfortranarray(g.uniform(-1, 1, (40, 50)))
    B = np.asfortranarray(g.uniform(-1, 1, (50, 30)))
    A[3, 7] = np.inf
    B[9, 4] = np.nan
    got, _ = _run(A, B, moduli=12)
    assert np.isnan(got[3, :]).all() and np.isnan(got[:, 4]).all()
    mask = np.ones_like(got, bool)
    mask[3, :] = False
    mask[:, 4] = False
    assert np.isfinite(got[mask]).all()
    ref = oracle.ozaki_crt_gemm(A, B, moduli=12)
    assert_bit_equal(got[mask], ref[mask])


def test_beta_zero_ignores_nan_c_and_zero_operands(cuda):
    g = np.random.default_rng(6)
    A = np.asfortranarray(g.uniform(-1, 1, (33, 44)))
    B = np.asfortranarray(g.uniform(-1, 1, (44, 55)))
    A[5, :] = 0.0
    C = np.full((33, 55), np.nan, order="F")
    got, _ = _run(A, B, C=C, moduli=10)
    assert np.isfinite(got).all()
    assert (got[5, :] == 0).all()
    assert_bit_equal(got, oracle.ozaki_crt_gemm(A, B, moduli=10))


def test_too_few_moduli_is_unsupported(cuda):
    d = torch.zeros((8, 1000), dtype=torch.float64, device=cuda)
    e = torch.zeros((1000, 8), dtype=torch.float64, device=cuda)
    c = torch.zeros((8, 8), dtype=torch.float64, device=cuda)
    with pytest.raises(gbblas.GBError) as err:
        gbblas.gemm_(c, d, e, mode="ozaki_crt", slices=1)
    assert err.value.status == gbblas._lib.GB_ERR_UNSUPPORTED


def _normwise_err(got, A, B, rows, cols):
    hi, lo, _ = oracle.dot2_entries(A, B, rows, cols)
    d = (got[rows, cols] - hi) - lo
    scale = np.sqrt(got.size / rows.size)
    return np.linalg.norm(d) * scale / (np.linalg.norm(A) * np.linalg.norm(B))


@pytest.mark.parametrize("dist", ["uniform", "ozaki"])
def test_accuracy_auto_beats_native(cuda, dist):
    M = K = N = 1024
    if dist == "uniform":
        A = workloads.uniform(M, K, stream=31)
        B = workloads.uniform(K, N, stream=32)
    else:
        A = workloads.ozaki_matrix(M, K, per="row", stream=31)
        B = workloads.ozaki_matrix(K, N, per="col", stream=32)
    oz, bound = _run(A, B, moduli=0, want_bound=True)
    Cn = torch.zeros((N, M), dtype=torch.float64, device=cuda).t()
    gbblas.gemm_(Cn, to_dev(A), to_dev(B), mode="native")
    nat = to_host(Cn)
    g = np.random.default_rng(2)
    rows, cols = g.integers(0, M, 4096), g.integers(0, N, 4096)
    e_oz = _normwise_err(oz, A, B, rows, cols)
    e_nat = _normwise_err(nat, A, B, rows, cols)
    assert e_oz <= bound <= 2.0 ** -50 * 1.0001
    assert e_oz <= e_nat, (e_oz, e_nat)


def test_bound_decreases_with_moduli_and_holds(cuda):
    M, K, N = 256, 2048, 256
    A = workloads.ozaki_matrix(M, K, per="row", stream=41)
    B = workloads.ozaki_matrix(K, N, per="col", stream=42)
    g = np.random.default_rng(3)
    rows, cols = g.integers(0, M, 2048), g.integers(0, N, 2048)
    prev = np.inf
    for n in (6, 9, 12, 15):
        got, bound = _run(A, B, moduli=n, want_bound=True)
        err = _normwise_err(got, A, B, rows, cols)
        assert err <= bound, (n, err, bound)
        assert bound < prev
        prev = bound


def test_8192_cubed_accuracy_beats_native(cuda):
    """M = N = K = 8192, sign*U[1,2)*2^(e_line + e_elem) inputs, moduli chosen by the library:
    normwise error (4096 Dot2-sampled entries) below the bound and below native FP64's."""
    n = 8192
    A = np.asfortranarray(workloads.ozaki_matrix(n, n, per="row", stream=1))
    B = np.asfortranarray(workloads.ozaki_matrix(n, n, per="col", stream=2))
    Ad, Bd = to_dev(A), to_dev(B)
    C = torch.empty((n, n), dtype=torch.float64, device=cuda).t()
    _, bound = gbblas.gemm_(C, Ad, Bd, mode="ozaki_crt", return_bound=True)
    oz = to_host(C)
    gbblas.gemm_(C, Ad, Bd, mode="native")
    nat = to_host(C)
    g = np.random.default_rng(12345)
    rows, cols = g.integers(0, n, 4096), g.integers(0, n, 4096)
    e_oz = _normwise_err(oz, A, B, rows, cols)
    e_nat = _normwise_err(nat, A, B, rows, cols)
    assert e_oz <= bound <= 2.0 ** -50
    assert e_oz <= e_nat, (e_oz, e_nat)


def test_automatic_call_captures_in_a_cuda_graph(cuda):
    """An automatic CRT call never waits on the host (the plan is chosen on the device), so
    it can be captured in a CUDA graph; replays equal the direct call bit for bit, also after
    the inputs change in place."""
    M, K, N = 384, 2048, 320
    A = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=71))
    B = np.asfortranarray(workloads.ozaki_matrix(K, N, per="col", stream=72))
    Ad, Bd = to_dev(A), to_dev(B)
    C_direct = torch.empty((N, M), dtype=torch.float64, device=cuda).t()
    gbblas.gemm_(C_direct, Ad, Bd, mode="ozaki_crt")       # warm-up outside the capture
    torch.cuda.synchronize()
    C_graph = torch.empty((N, M), dtype=torch.float64, device=cuda).t()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        gbblas.gemm_(C_graph, Ad, Bd, mode="ozaki_crt")
    graph.replay()
    torch.cuda.synchronize()
    assert_bit_equal(to_host(C_graph), to_host(C_direct))
    A2 = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=73))
    Ad.copy_(to_dev(A2))
    graph.replay()
    gbblas.gemm_(C_direct, Ad, Bd, mode="ozaki_crt")
    torch.cuda.synchronize()
    gbblas.check_device_status()
    assert_bit_equal(to_host(C_graph), to_host(C_direct))


@pytest.mark.parametrize("tb", [0, 1])
def test_leading_dimensions_larger_than_rows(cuda, tb):
    """Operands inside larger column-major buffers (lda > M, ldb > rows of B as stored, ldc > M):
    the same bits as packed operands, and C's padding rows are not written."""
    from gpu_util import to_dev_ld
    M, K, N = 150, 333, 97
    g = np.random.default_rng(404 + tb)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-6, 7, (M, K))))
    Bl = g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-6, 7, (K, N)))
    B = np.asfortranarray(Bl.T if tb else Bl)
    Ad, _ = to_dev_ld(A, M + 13)
    Bd, _ = to_dev_ld(B, B.shape[0] + 7)
    Cd, Cbuf = to_dev_ld(np.zeros((M, N)), M + 5, fill=3.0)
    gbblas.gemm_raw(0, tb, M, N, K, 1.0, Ad.data_ptr(), M + 13, Bd.data_ptr(), B.shape[0] + 7, 0.0,
                    Cd.data_ptr(), M + 5, dtype=torch.float64, mode=gbblas.MODE_OZAKI_CRT, slices=15,
                    stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    assert_bit_equal(to_host(Cd), oracle.ozaki_crt_gemm(A, Bl, moduli=15))
    assert np.all(to_host(Cbuf)[M:, :N] == 3.0)
