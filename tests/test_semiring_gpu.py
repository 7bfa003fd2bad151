"""GPU parity of the semiring GEMM (C ABI through ctypes) against the oracle.

Every semiring's (+) is min or max and every (x) rounds once, so each output element is
independent of the K order: all checks are bit-exact (NaN positions compared as
positions), including signed zeros, infinities, subnormals and int32 wrap-around.
"""
import ctypes
import os

import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib
import oracle
from gpu_util import assert_bit_equal, to_dev, to_dev_ld, to_host

pytestmark = pytest.mark.gpu

DTYPES = {np.float64: torch.float64, np.float32: torch.float32, np.int32: torch.int32}
SHAPES = [(1, 1, 1), (7, 9, 5), (130, 70, 33), (129, 257, 17), (300, 200, 1000), (64, 256, 8)]


def operands(g, dt, M, K, N, special=True):
    if np.dtype(dt).kind == "i":
        A = g.integers(-2**31, 2**31, (M, K)).astype(dt)
        B = g.integers(-2**31, 2**31, (K, N)).astype(dt)
        if special and M > 1 and K > 1:
            A[0, :] = 2**31 - 1
            A[1, :] = -2**31
        return A, B
    A = g.uniform(-2, 2, (M, K)).astype(dt)
    B = g.uniform(-2, 2, (K, N)).astype(dt)
    if special and M > 6 and K > 6 and N > 3:
        A[0, 0] = np.nan
        A[1, :] = -0.0
        B[:, 2] = 0.0
        A[2, 3] = np.inf
        B[3, 1] = -np.inf
        A[4, :] = np.nan
        A[5, 5] = np.finfo(dt).tiny / 4
        B[6 % K, :] = -0.0
    return A, B


def run(sr, A, B, dt, C0=None, accumulate=False, trans=(False, False), rowmajor_c=False):
    M, N = A.shape[0], B.shape[1]
    tdt = DTYPES[dt]
    Ad = to_dev(A.T).t() if trans[0] else to_dev(A)
    Bd = to_dev(B.T).t() if trans[1] else to_dev(B)
    if C0 is not None:
        Cd = torch.from_numpy(np.ascontiguousarray(C0)).cuda() if rowmajor_c else to_dev(C0)
    elif rowmajor_c:
        Cd = torch.empty((M, N), dtype=tdt, device="cuda")
    else:
        Cd = torch.empty((N, M), dtype=tdt, device="cuda").t()
    out = gbblas.gemm_semiring_(Cd, Ad, Bd, sr, accumulate=accumulate)
    assert out is Cd
    torch.cuda.synchronize()
    gbblas.check_device_status()
    return to_host(Cd)


@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
@pytest.mark.parametrize("sr", oracle.SEMIRINGS)
@pytest.mark.parametrize("dt", list(DTYPES), ids=["f64", "f32", "i32"])
def test_semiring_matches_oracle(dt, sr, shape):
    M, K, N = shape
    g = np.random.default_rng(M * 131 + K * 7 + N)
    A, B = operands(g, dt, M, K, N)
    assert_bit_equal(run(sr, A, B, dt), oracle.semiring_gemm(A, B, sr, dtype=dt))


@pytest.mark.parametrize("trans", [(False, True), (True, False), (True, True)], ids=["NT", "TN", "TT"])
@pytest.mark.parametrize("sr", ["min_plus", "max_times"])
@pytest.mark.parametrize("dt", list(DTYPES), ids=["f64", "f32", "i32"])
def test_semiring_transposes(dt, sr, trans):
    g = np.random.default_rng(11)
    A, B = operands(g, dt, 133, 71, 95)
    assert_bit_equal(run(sr, A, B, dt, trans=trans), oracle.semiring_gemm(A, B, sr, dtype=dt))


@pytest.mark.parametrize("sr", oracle.SEMIRINGS)
@pytest.mark.parametrize("dt", list(DTYPES), ids=["f64", "f32", "i32"])
def test_semiring_accumulate(dt, sr):
    g = np.random.default_rng(5)
    A, B = operands(g, dt, 70, 40, 50)
    C0, _ = operands(g, dt, 70, 50, 1, special=False)
    if np.dtype(dt).kind == "f":
        C0[3, :] = np.nan
        C0[4, :] = -0.0
    ref = oracle.semiring_gemm(A, B, sr, C=C0, accumulate=True, dtype=dt)
    assert_bit_equal(run(sr, A, B, dt, C0=C0, accumulate=True), ref)
    # row-major C (computed as C^T = B^T (x) A^T)
    assert_bit_equal(run(sr, A, B, dt, C0=C0, accumulate=True, rowmajor_c=True), ref)


@pytest.mark.parametrize("sr", oracle.SEMIRINGS)
@pytest.mark.parametrize("dt", list(DTYPES), ids=["f64", "f32", "i32"])
def test_semiring_empty_contraction_gives_identity(dt, sr):
    A = np.zeros((5, 0), dtype=dt)
    B = np.zeros((0, 4), dtype=dt)
    assert_bit_equal(run(sr, A, B, dt), oracle.semiring_gemm(A, B, sr, dtype=dt))
    C0 = np.arange(20, dtype=dt).reshape(5, 4) - 7
    assert_bit_equal(run(sr, A, B, dt, C0=C0, accumulate=True),
                     oracle.semiring_gemm(A, B, sr, C=C0, accumulate=True, dtype=dt))


def test_semiring_leading_dimensions():
    g = np.random.default_rng(3)
    A, B = operands(g, np.float32, 45, 30, 20)
    Ad, _ = to_dev_ld(A, 64)
    Bd, _ = to_dev_ld(B, 40)
    Cd, Cbuf = to_dev_ld(np.zeros((45, 20), np.float32), 48, fill=7.0)
    gbblas.gemm_semiring_(Cd, Ad, Bd, "max_plus")
    torch.cuda.synchronize()
    assert_bit_equal(to_host(Cd), oracle.semiring_gemm(A, B, "max_plus", dtype=np.float32))
    pad = to_host(Cbuf)[45:, :20]
    assert np.all(pad == 7.0), "writes outside the M x N block"


@pytest.mark.parametrize("dt", list(DTYPES), ids=["f64", "f32", "i32"])
def test_semiring_apsp_fixture(dt):
    """(min, +) closure of a 48-node digraph by repeated squaring on the GPU equals the
    committed Floyd-Warshall distances."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "semiring", "apsp_48.npz"))
    W, Dref = z["W"], z["D"]
    inf_i = 2**29
    X = np.where(np.isinf(W), inf_i, W).astype(dt) if dt == np.int32 else W.astype(dt)
    Xd = to_dev(X)
    for _ in range(6):
        Yd = torch.empty_like(Xd.t().contiguous()).t()
        gbblas.gemm_semiring_(Yd, Xd, Xd, "min_plus")
        Xd = Yd
    X = to_host(Xd)
    got = np.where(X >= inf_i, np.inf, X).astype(np.float64) if dt == np.int32 else X.astype(np.float64)
    assert np.array_equal(got, Dref)


@pytest.mark.parametrize("sr", ["min_plus", "max_min"])
@pytest.mark.parametrize("dt", [np.float32, np.int32], ids=["f32", "i32"])
def test_semiring_large_sampled(dt, sr):
    """2048 x 2048 x 2048: the rows and columns of 48 sampled outputs each, against the oracle."""
    M = N = K = 2048
    tdt = DTYPES[dt]
    gen = torch.Generator(device="cuda").manual_seed(17)
    if dt == np.int32:
        Ad = torch.randint(-10**6, 10**6, (K, M), dtype=tdt, device="cuda", generator=gen).t()
        Bd = torch.randint(-10**6, 10**6, (N, K), dtype=tdt, device="cuda", generator=gen).t()
    else:
        Ad = (torch.rand((K, M), dtype=tdt, device="cuda", generator=gen) * 200 - 100).t()
        Bd = (torch.rand((N, K), dtype=tdt, device="cuda", generator=gen) * 200 - 100).t()
    Cd = torch.empty((N, M), dtype=tdt, device="cuda").t()
    gbblas.gemm_semiring_(Cd, Ad, Bd, sr)
    torch.cuda.synchronize()
    g = np.random.default_rng(2)
    rows = np.sort(g.choice(M, 48, replace=False))
    cols = np.sort(g.choice(N, 48, replace=False))
    A = to_host(Ad[torch.as_tensor(rows, device="cuda"), :])
    B = to_host(Bd[:, torch.as_tensor(cols, device="cuda")])
    ref = oracle.semiring_gemm(A, B, sr, dtype=dt)
    got = to_host(Cd)[np.ix_(rows, cols)]
    assert_bit_equal(np.asfortranarray(got), ref)


def test_semiring_launches_are_counted():
    before = gbblas.launch_counts().get("semiring_gemm", 0)
    A = to_dev(np.ones((8, 8), np.float32))
    gbblas.gemm_semiring(A, A, "min_plus")
    torch.cuda.synchronize()
    assert gbblas.launch_counts()["semiring_gemm"] == before + 1


def test_semiring_argument_errors():
    L = _lib.lib()
    A = torch.zeros((4, 4), dtype=torch.float32, device="cuda").t()
    p = ctypes.c_void_p(A.data_ptr())
    st = ctypes.c_void_p(0)
    assert L.gb_gemm_semiring_f32(5, 0, 0, 4, 4, 4, p, 4, p, 4, 0, p, 4, st) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_gemm_semiring_f32(-1, 0, 0, 4, 4, 4, p, 4, p, 4, 0, p, 4, st) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_gemm_semiring_f32(0, 0, 0, 4, 4, 4, p, 4, p, 4, 2, p, 4, st) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_gemm_semiring_f32(0, 0, 0, 4, 4, 4, p, 3, p, 4, 0, p, 4, st) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_gemm_semiring_f32(0, 2, 0, 4, 4, 4, p, 4, p, 4, 0, p, 4, st) == _lib.GB_ERR_INVALID_VALUE
    with pytest.raises(ValueError):
        gbblas.gemm_semiring_(A, A, A, "plus_times")
    with pytest.raises(TypeError):
        gbblas.gemm_semiring_(A, A.double(), A, "min_plus")
    with pytest.raises(TypeError):
        h = A.half()
        gbblas.gemm_semiring_(h, h, h, "min_plus")
    with pytest.raises(gbblas.DimensionMismatch):
        gbblas.gemm_semiring_(A, A[:, :3], A, "min_plus")
