"""Property-based checks of the oracle restatements (random shapes and values, including
signed zeros, infinities, NaN and wide exponent ranges): the restatements agree with their
independent pins for every drawn case, not only the fixed fixtures.  CPU only."""
from fractions import Fraction

import numpy as np
import pytest

import oracle

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings, strategies as st  # noqa: E402
from hypothesis.extra import numpy as hnp  # noqa: E402

SETTINGS = settings(max_examples=60, deadline=None, derandomize=True)

finite64 = st.floats(min_value=-1e6, max_value=1e6, allow_nan=False, allow_infinity=False, width=64)
special64 = st.one_of(finite64, st.sampled_from([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -2.5e-310]))


def matrices(rows, cols, elements, dtype=np.float64):
    return hnp.arrays(dtype, st.tuples(st.just(rows), st.just(cols)), elements=elements)


@st.composite
def semiring_case(draw):
    M = draw(st.integers(1, 6))
    K = draw(st.integers(0, 7))
    N = draw(st.integers(1, 6))
    dt = draw(st.sampled_from([np.float64, np.float32, np.int32]))
    if dt == np.int32:
        el = st.integers(-2**31, 2**31 - 1)
    elif dt == np.float32:
        el = st.one_of(st.floats(-1e4, 1e4, width=32), st.sampled_from([0.0, -0.0, np.inf, -np.inf, np.nan]))
    else:
        el = special64
    A = draw(matrices(M, K, el, dt))
    B = draw(matrices(K, N, el, dt))
    sr = draw(st.sampled_from(oracle.SEMIRINGS))
    return A, B, sr, dt


def _same(x, y):
    x, y = np.ascontiguousarray(x), np.ascontiguousarray(y)
    if x.dtype.kind == "i":
        return np.array_equal(x, y)
    nx, ny = np.isnan(x), np.isnan(y)
    u = np.uint64 if x.dtype == np.float64 else np.uint32
    return np.array_equal(nx, ny) and np.array_equal(np.where(nx, 0, x).view(u), np.where(ny, 0, y).view(u))


@SETTINGS
@given(semiring_case())
def test_semiring_fold_equals_reduction_and_reversed_order(case):
    A, B, sr, dt = case
    seq = oracle.semiring_gemm(A, B, sr, dtype=dt)
    assert _same(seq, oracle.semiring_gemm_reduce(A, B, sr, dtype=dt))
    assert _same(seq, oracle.semiring_gemm(A[:, ::-1], B[::-1, :], sr, dtype=dt))


@st.composite
def chain_case(draw):
    M = draw(st.integers(1, 4))
    K = draw(st.integers(1, 9))
    P = draw(st.integers(1, 4))
    el = st.one_of(st.floats(-1e3, 1e3, allow_nan=False, width=64), st.sampled_from([0.0, -0.0, 1e-310, -3e-320]))
    return draw(matrices(M, K, el)), draw(matrices(K, P, el))


@SETTINGS
@given(chain_case())
def test_c_chain_equals_exact_rational_chain(case):
    """jmul!'s FMA chain in C equals the exact-rational restatement bit for bit (signed zeros,
    subnormals, cancellation)."""
    A, X = case
    A, X = np.asfortranarray(A), np.asfortranarray(X)
    got = oracle.jmul(A, X)
    ref = oracle.chain_exact(A, X)
    assert np.array_equal(got.view(np.uint64), np.asfortranarray(ref).view(np.uint64))


@SETTINGS
@given(chain_case(), st.data())
def test_kernel_chain_equals_exact_rational_chain(case, data):
    """kernel! (the chain folded onto D's value) equals the exact-rational chain started from D."""
    A, X = case
    M, K = A.shape
    P = X.shape[1]
    D0 = data.draw(matrices(M, P, st.floats(-1e3, 1e3, allow_nan=False, width=64)))
    got = oracle.kernel_chain(np.asfortranarray(D0).ravel(order="F"), np.asfortranarray(A).ravel(order="F"),
                              np.asfortranarray(X).ravel(order="F"), M, P, M, K, K)
    ref = oracle.chain_exact(A, X, D0=D0)
    assert np.array_equal(got.view(np.uint64), np.asfortranarray(ref).ravel(order="F").view(np.uint64))


@st.composite
def crt_case(draw):
    M = draw(st.integers(1, 4))
    K = draw(st.integers(1, 24))
    N = draw(st.integers(1, 4))
    moduli = draw(st.integers(10, 20))
    mant = st.floats(-1.0, 1.0, allow_nan=False, width=64)
    A = draw(matrices(M, K, mant)) * np.ldexp(1.0, draw(hnp.arrays(np.int64, (M, K), elements=st.integers(-20, 20))))
    B = draw(matrices(K, N, mant)) * np.ldexp(1.0, draw(hnp.arrays(np.int64, (K, N), elements=st.integers(-20, 20))))
    return np.asfortranarray(A), np.asfortranarray(B), moduli


@SETTINGS
@given(crt_case())
def test_crt_restatement_is_the_rounded_exact_integer_product(case):
    """For any shape, value and moduli count: the CRT restatement equals the exact integer
    product of the t-bit operands (Python rationals), rounded once to FP64 and rescaled."""
    A, B, moduli = case
    M, K = A.shape
    N = B.shape[1]
    t = oracle.crt_bits_for(K, moduli)
    if t < 1:
        return
    C = oracle.ozaki_crt_gemm(A, B, moduli=moduli)
    Ya, ea = oracle._fixed_rows(A, t)
    Yb, eb = oracle._fixed_rows(B.T, t)
    for i in range(M):
        for j in range(N):
            exact_int = sum(int(Ya[i, k]) * int(Yb[j, k]) for k in range(K))
            want = float(Fraction(exact_int) * Fraction(2) ** int(ea[i] + eb[j] - 2 * t))
            assert C[i, j] == want or (C[i, j] == 0 and want == 0)
