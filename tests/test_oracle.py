"""CPU checks of the oracle itself: golden fixtures, restatements against each other."""
import glob
import os
from fractions import Fraction

import numpy as np
import pytest

import oracle

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 10


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_c_oracle_matches_golden_bit_exact(path):
    z = np.load(path)
    A, X, D = z["A"], z["X"], z["D"]
    got = oracle.jmul(A, X, dtype=D.dtype.type)
    assert got.dtype == D.dtype
    np.testing.assert_array_equal(got.view(np.uint64 if D.dtype == np.float64 else np.uint32),
                                  np.asfortranarray(D).view(np.uint64 if D.dtype == np.float64 else np.uint32))


def test_exact_chain_reproduces_a_fixture():
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "f64_13x12x12_uniform.npz"))
    D = oracle.chain_exact(z["A"], z["X"])
    np.testing.assert_array_equal(D, z["D"])


TILES = {np.float64: [(40, 5), (12, 4), (10, 5), (20, 5), (16, 14), (8, 6)],
         np.float32: [(80, 5), (24, 4), (20, 5), (40, 5), (16, 14)]}


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("shape", [(1, 1, 1), (7, 5, 3), (41, 17, 13), (64, 64, 64), (130, 70, 33)])
@pytest.mark.parametrize("nthreads", [1, 4])
def test_tiled_baseline_equals_chain(dtype, shape, nthreads):
    """Every instantiated register tile (and the host's own) gives jmul!'s chain bit for bit."""
    M, K, N = shape
    g = np.random.default_rng(5)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)).astype(dtype))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)).astype(dtype))
    ref = oracle.gemm(A, B, dtype=dtype)
    for tile in [None] + TILES[dtype]:
        got = oracle.jmul_tiled(A, B, nthreads=nthreads, dtype=dtype, tile=tile)
        np.testing.assert_array_equal(got, ref)


# (t_size, register bytes, register count) -> (elements per register, rows, cols)
PICK_KERNEL_SIZE = [
    ((8, 64, 32), (8, 40, 5)),    # AVX-512, Float64
    ((4, 64, 32), (16, 80, 5)),   # AVX-512, Float32
    ((8, 32, 16), (4, 12, 4)),    # AVX2, Float64
    ((4, 32, 16), (8, 24, 4)),    # AVX2, Float32
    ((8, 16, 32), (2, 10, 5)),    # 128-bit NEON (32 registers), Float64
    ((4, 16, 32), (4, 20, 5)),    # 128-bit NEON, Float32
    ((8, 32, 32), (4, 20, 5)),    # 32 registers of 4 Float64 lanes
]


@pytest.mark.parametrize("args,expect", PICK_KERNEL_SIZE, ids=["avx512_f64", "avx512_f32", "avx2_f64",
                                                              "avx2_f32", "neon_f64", "neon_f32", "32x4_f64"])
def test_pick_kernel_size_restatement(args, expect):
    """The greedy search of src/kernel_structure.jl:76-99, in Python and in the C oracle."""
    assert oracle.pick_kernel_size(*args) == expect
    import ctypes
    r, c = ctypes.c_int(0), ctypes.c_int(0)
    epr = oracle.lib().or_pick_kernel_size(*args, ctypes.byref(r), ctypes.byref(c))
    assert (epr, r.value, c.value) == expect


def test_host_tile_is_instantiated():
    for dt in (np.float64, np.float32):
        assert oracle.host_tile(dt) in TILES[dt]


def test_time_jmul_tiled_reference_shape():
    """The timing helper runs the reference's benchmark shape (D 16x14 = A 16x32 * X 32x14)."""
    g = np.random.default_rng(8)
    A = np.asfortranarray(g.standard_normal((16, 32)))
    X = np.asfortranarray(g.standard_normal((32, 14)))
    for tile in (None, (16, 14)):
        ns = oracle.time_jmul_tiled(A, X, tile=tile, reps=100, batches=3)
        assert 0 < ns < 1e7


def test_chain_entries_equals_full_oracle():
    g = np.random.default_rng(6)
    A = np.asfortranarray(g.uniform(-1, 1, (33, 20)))
    B = np.asfortranarray(g.uniform(-1, 1, (25, 20)))   # stored N x K: op(B) = B^T
    C = np.asfortranarray(g.uniform(-1, 1, (33, 25)))
    full = oracle.gemm(A, B, C=C, alpha=1.5, beta=0.5, trans_b=True)
    rows = g.integers(0, 33, 50)
    cols = g.integers(0, 25, 50)
    got = oracle.chain_entries(A, B, rows, cols, C=C, alpha=1.5, beta=0.5, trans_b=True)
    np.testing.assert_array_equal(got, full[rows, cols])


def test_alpha_beta_semantics():
    A = np.asfortranarray(np.ones((3, 2)))
    B = np.asfortranarray(np.ones((2, 4)))
    C = np.asfortranarray(np.full((3, 4), np.nan))
    out = oracle.gemm(A, B, C=C, alpha=2.0, beta=0.0)   # beta == 0: C is not read
    assert np.all(out == 4.0)
    C2 = np.asfortranarray(np.full((3, 4), 3.0))
    A2 = np.asfortranarray(np.full((3, 2), np.nan))
    out = oracle.gemm(A2, B, C=C2, alpha=0.0, beta=2.0)  # alpha == 0: A, B are not read
    assert np.all(out == 6.0)
    out = oracle.gemm(np.zeros((3, 0), order="F"), np.zeros((0, 4), order="F"), C=C2, alpha=1.0, beta=0.5)
    assert np.all(out == 1.5)


def test_dot2_is_near_exact():
    g = np.random.default_rng(7)
    K = 300
    A = np.asfortranarray(g.standard_normal((4, K)) * np.ldexp(1.0, g.integers(-20, 20, (4, K))))
    B = np.asfortranarray(g.standard_normal((K, 3)))
    rows = np.array([0, 1, 2, 3])
    cols = np.array([0, 1, 2, 0])
    hi, lo, ab = oracle.dot2_entries(A, B, rows, cols)
    for s in range(4):
        exact = sum(Fraction(A[rows[s], k]) * Fraction(B[k, cols[s]]) for k in range(K))
        err = abs(Fraction(hi[s]) + Fraction(lo[s]) - exact)
        assert float(err) <= 4 * 2.0 ** -104 * ab[s] + 2.0 ** -1000


def test_ozaki_split_reconstructs():
    g = np.random.default_rng(8)
    X = g.standard_normal((20, 50)) * np.ldexp(1.0, g.integers(-8, 9, (20, 50)))
    X[3] = 0.0
    for bits in (5, 6, 7, 9):
        for s in (1, 3, 8, 12):
            d, e = oracle.ozaki_split(X, s, bits)
            assert np.all(np.abs(d) <= 2 ** (bits - 1))
            assert np.all(d[1:] < 2 ** (bits - 1))
            assert np.all(d == np.rint(d))
            w = 2.0 ** (1 - bits * np.arange(1, s + 1))
            rec = np.ldexp(np.tensordot(w, d, axes=1), e[:, None])
            err = np.abs(rec - X)
            assert np.all(err <= np.ldexp(1.0, e - s * bits)[:, None] * (1 + 1e-12))


def test_ozaki_restatement_error_within_truncation():
    g = np.random.default_rng(9)
    M, K, N = 12, 200, 9
    A = g.uniform(-1, 1, (M, K))
    B = g.uniform(-1, 1, (K, N))
    exact = oracle.gemm(A, B)
    prev = None
    for s in (2, 4, 6, 8):
        got = oracle.ozaki_gemm(A, B, slices=s)
        err = np.linalg.norm(got - exact) / (np.linalg.norm(A) * np.linalg.norm(B))
        if prev is not None:
            assert err <= prev * 1.01 + 1e-17
        prev = err
    assert prev < 1e-15


def test_ozaki_plan_grouping_respects_exactness():
    for K in (1, 64, 1000, 4096, 8192, 16384, 100000):
        for s in (1, 5, 9, 14):
            p = oracle.ozaki_plan(K, s)
            assert p["products"] == sum(1 for a in range(1, s + 1) for b in range(1, s + 1) if a + b <= s + 1)
            for level, pairs in p["groups"]:
                assert all(a + b + 2 == level for a, b in pairs)
                assert len(pairs) * p["k_chunk"] * 2.0 ** (2 * p["bits"] - 2) <= 2.0 ** 24


def test_crt_restatement_against_exact_rationals():
    """The CRT-mode restatement: exact integer product of the t-bit operands, rounded once
    to FP64 (checked here with Python rationals), and its error small against the exact
    product of the unrounded inputs."""
    from fractions import Fraction
    g = np.random.default_rng(8)
    A = g.uniform(-1, 1, (9, 40)) * np.ldexp(1.0, g.integers(-6, 7, (9, 40)))
    B = g.uniform(-1, 1, (40, 7)) * np.ldexp(1.0, g.integers(-6, 7, (40, 7)))
    t = oracle.crt_bits_for(40, 16)
    C = oracle.ozaki_crt_gemm(A, B, moduli=16)
    Ya, ea = oracle._fixed_rows(A, t)
    Yb, eb = oracle._fixed_rows(B.T, t)
    for i in range(9):
        for j in range(7):
            exact_int = sum(int(Ya[i, k]) * int(Yb[j, k]) for k in range(40))
            assert C[i, j] == float(Fraction(exact_int) * Fraction(2) ** int(ea[i] + eb[j] - 2 * t))
            exact = sum(Fraction(A[i, k]) * Fraction(B[k, j]) for k in range(40))
            scale = float(np.abs(A[i]).max() * np.abs(B[:, j]).max())
            assert abs(float(Fraction(C[i, j]) - exact)) <= 40 * scale * 2.0 ** -t + 2.0 ** -52 * abs(C[i, j])


def test_crt_moduli_pairwise_coprime():
    import math
    m = oracle.crt_moduli(20)
    assert m[0] == 253 and len(set(m)) == 20 and max(m) <= 253
    assert all(math.gcd(a, b) == 1 for i, a in enumerate(m) for b in m[i + 1:])


# ---------------------------------------------------------------------------- semirings
SEMIRING_FIXTURE = os.path.join(os.path.dirname(__file__), "golden", "semiring", "apsp_48.npz")


def _special_operands(g, dt, M, K, N):
    if np.dtype(dt).kind == "i":
        A = g.integers(-2**31, 2**31, (M, K)).astype(dt)
        B = g.integers(-2**31, 2**31, (K, N)).astype(dt)
        return A, B
    A = g.uniform(-2, 2, (M, K)).astype(dt)
    B = g.uniform(-2, 2, (K, N)).astype(dt)
    A[0, 0] = np.nan
    A[1, :] = -0.0
    B[:, 2] = 0.0
    A[2, 3] = np.inf
    B[3, 1] = -np.inf
    A[4, :] = np.nan
    A[5, 5] = np.finfo(dt).tiny / 4     # subnormal
    return A, B


def _same(x, y):
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    if x.dtype.kind == "i":
        return np.array_equal(x, y)
    nx, ny = np.isnan(x), np.isnan(y)
    u = np.uint64 if x.dtype == np.float64 else np.uint32
    return np.array_equal(nx, ny) and np.array_equal(np.where(nx, 0, x).view(u), np.where(ny, 0, y).view(u))


@pytest.mark.parametrize("dt", [np.float64, np.float32, np.int32])
@pytest.mark.parametrize("sr", oracle.SEMIRINGS)
def test_semiring_sequential_equals_reduction(dt, sr):
    """The K-ordered fold and numpy's pairwise reduction give the same bits (NaN, +-0, Inf)."""
    g = np.random.default_rng(7)
    A, B = _special_operands(g, dt, 9, 11, 6)
    assert _same(oracle.semiring_gemm(A, B, sr, dtype=dt), oracle.semiring_gemm_reduce(A, B, sr, dtype=dt))
    # a reversed K order gives the same bits too
    assert _same(oracle.semiring_gemm(A, B, sr, dtype=dt), oracle.semiring_gemm(A[:, ::-1], B[::-1, :], sr, dtype=dt))


def test_semiring_identities_and_wrap():
    e = np.zeros((3, 0))
    f = np.zeros((0, 2))
    assert np.all(oracle.semiring_gemm(e, f, "min_plus") == np.inf)
    assert np.all(oracle.semiring_gemm(e, f, "max_times") == -np.inf)
    ei, fi = e.astype(np.int32), f.astype(np.int32)
    assert np.all(oracle.semiring_gemm(ei, fi, "min_max", dtype=np.int32) == 2**31 - 1)
    assert np.all(oracle.semiring_gemm(ei, fi, "max_plus", dtype=np.int32) == -2**31)
    big = np.array([[2**31 - 1]], dtype=np.int32)
    one = np.array([[1]], dtype=np.int32)
    assert oracle.semiring_gemm(big, one, "max_plus", dtype=np.int32)[0, 0] == -2**31   # wraps
    z = oracle.semiring_gemm(np.array([[-0.0]]), np.array([[-0.0]]), "min_plus")
    assert z[0, 0] == 0 and not np.signbit(z[0, 0])                                      # +0.0


def test_semiring_fixture_is_floyd_warshall():
    """The committed APSP fixture equals Floyd-Warshall recomputed here in Python integers."""
    z = np.load(SEMIRING_FIXTURE)
    W = [[None if not np.isfinite(v) or i == j else int(v) for j, v in enumerate(row)]
         for i, row in enumerate(z["W"])]
    D = oracle.floyd_warshall(W)
    assert np.array_equal(np.array([[np.inf if v is None else v for v in r] for r in D]), z["D"])


@pytest.mark.parametrize("dt", [np.float64, np.float32, np.int32])
def test_semiring_min_plus_closure_is_apsp(dt):
    """Repeated (min, +) squaring of the weight matrix reproduces the fixture's distances."""
    z = np.load(SEMIRING_FIXTURE)
    W, Dref = z["W"], z["D"]
    inf_i = 2**29      # int32 "no edge": sums of two stay below 2^31
    X = np.where(np.isinf(W), inf_i, W).astype(dt) if dt == np.int32 else W.astype(dt)
    for _ in range(6):   # 2^6 >= 47 edges
        X = oracle.semiring_gemm(X, X, "min_plus", dtype=dt)
    got = np.where(X >= inf_i, np.inf, X).astype(np.float64) if dt == np.int32 else X.astype(np.float64)
    assert np.array_equal(got, Dref)


def test_quad_is_near_exact_and_agrees_with_dot2():
    """The binary128 dot product: within K 2^-113 sum|a||b| (+ double-double rounding) of the
    exact rational value, and equal to Dot2 within Dot2's error bound."""
    g = np.random.default_rng(17)
    K = 400
    A = np.asfortranarray(g.standard_normal((5, K)) * np.ldexp(1.0, g.integers(-30, 30, (5, K))))
    B = np.asfortranarray(g.standard_normal((K, 4)) * np.ldexp(1.0, g.integers(-30, 30, (K, 4))))
    rows = np.array([0, 1, 2, 3, 4, 0])
    cols = np.array([0, 1, 2, 3, 0, 3])
    qhi, qlo = oracle.quad_entries(A, B, rows, cols)
    dhi, dlo, ab = oracle.dot2_entries(A, B, rows, cols)
    for s in range(rows.size):
        exact = sum(Fraction(A[rows[s], k]) * Fraction(B[k, cols[s]]) for k in range(K))
        err = abs(Fraction(qhi[s]) + Fraction(qlo[s]) - exact)
        assert float(err) <= K * 2.0 ** -113 * ab[s] + 2.0 ** -105 * abs(float(exact)) + 2.0 ** -1000
        u = 2.0 ** -53   # Dot2's bound: u^2 |x| + gamma_K^2 sum|a||b|
        assert abs((dhi[s] - qhi[s]) + (dlo[s] - qlo[s])) <= 2 * (K * u) ** 2 * ab[s] + 2.0 ** -104 * abs(qhi[s])
    # transposed operands address the same values
    qt, _ = oracle.quad_entries(np.asfortranarray(A.T), np.asfortranarray(B.T), rows, cols, trans_a=True,
                                trans_b=True)
    assert np.array_equal(qt, qhi)


@pytest.mark.parametrize("dtype,bits", [(np.float64, 53), (np.float32, 24)])
@pytest.mark.parametrize("init", [False, True])
def test_kernel_chain_matches_exact_restatement(dtype, bits, init):
    """kernel! / initkernel! on strided buffers (A and D share stride_AD) equal the exact-rational
    chain started from D's value (kernel!) or from the rounded first product (initkernel!)."""
    g = np.random.default_rng(23 + int(init))
    Mk, Pk, N, sAD, sX = 7, 5, 9, 10, 12
    Abuf = g.standard_normal(sAD * N).astype(dtype)
    Xbuf = g.standard_normal(sX * Pk).astype(dtype)
    Dbuf = g.standard_normal(sAD * Pk).astype(dtype)
    Abuf[3] = -0.0
    Dbuf[sAD + 1] = -0.0
    out = oracle.kernel_chain(Dbuf, Abuf, Xbuf, Mk, Pk, sAD, sX, N, init=init, dtype=dtype)
    A = Abuf.reshape(N, sAD).T[:Mk, :N].astype(np.float64)
    X = Xbuf.reshape(Pk, sX).T[:N, :Pk].astype(np.float64)
    D0 = Dbuf.reshape(Pk, sAD).T[:Mk, :Pk].astype(np.float64)
    ref = oracle.chain_exact(A, X, bits=bits, D0=None if init else D0).astype(dtype)
    got = out.reshape(Pk, sAD).T[:Mk, :Pk]
    assert np.array_equal(got.view(np.uint64 if dtype == np.float64 else np.uint32),
                          np.asarray(ref, order="C").view(np.uint64 if dtype == np.float64 else np.uint32))
    # padding rows between the tiles are untouched
    assert np.array_equal(out.reshape(Pk, sAD)[:, Mk:], Dbuf.reshape(Pk, sAD)[:, Mk:])
