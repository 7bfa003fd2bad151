"""GPU parity of jBLAS's pointer-level micro-kernels, kernel! and initkernel!
(src/kernels.jl:212-273), through the C ABI (gb_kernel_f64/_f32) against the oracle.

kernel! folds A*X onto D's value in an FMA chain (d = fma(a_n, x_n, d), n = 1..N), which rounds
differently from a BLAS beta = 1 update; both modes are bit-exact against the C restatement.
"""
import ctypes

import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib
import oracle

pytestmark = pytest.mark.gpu

TORCH = {np.float64: torch.float64, np.float32: torch.float32}


def buffers(g, dtype, Mk, Pk, N, sAD, sX, special=False):
    A = g.standard_normal(sAD * max(N, 1)).astype(dtype)
    X = g.standard_normal(sX * Pk).astype(dtype)
    D = g.standard_normal(sAD * Pk).astype(dtype)
    if special and Mk > 4 and N > 3:
        A[0] = -0.0                      # (-0) * x onto -0 keeps -0 only when every term is -0
        D[0] = -0.0
        A[1 + sAD] = np.inf
        X[2] = np.nan
        D[3] = np.inf
    return D, A, X


def run(D, A, X, Mk, Pk, sAD, sX, N, init, dtype):
    dev = {k: torch.from_numpy(v.copy()).cuda() for k, v in (("D", D), ("A", A), ("X", X))}
    gbblas.kernel_raw(dev["D"].data_ptr(), dev["A"].data_ptr(), dev["X"].data_ptr(), Mk, Pk, sAD, sX, N,
                      dtype=TORCH[dtype], init=init, stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return dev["D"].cpu().numpy()


def same_bits(got, ref):
    u = np.uint64 if got.dtype == np.float64 else np.uint32
    nan_g, nan_r = np.isnan(got), np.isnan(ref)
    assert np.array_equal(nan_g, nan_r), "NaN positions differ"
    bad = ~nan_g & (got.view(u) != ref.view(u))
    assert not bad.any(), "%d mismatches, first at %s" % (bad.sum(), np.argwhere(bad)[:3].ravel().tolist())


# (Mk, Pk, N, stride_AD, stride_X): the reference's AVX-512 micro-tiles (f64 40x5, f32 80x5 from
# pick_kernel_size, src/kernel_structure.jl:76-99), small and ragged tiles, and large products
CASES = [(40, 5, 64, 48, 70), (80, 5, 300, 80, 300), (8, 4, 1, 8, 1), (1, 1, 7, 1, 9), (33, 17, 129, 40, 130),
         (1000, 700, 513, 1003, 520), (130, 2100, 64, 130, 64)]


@pytest.mark.parametrize("init", [False, True], ids=["kernel", "initkernel"])
@pytest.mark.parametrize("case", CASES, ids=["x".join(map(str, c)) for c in CASES])
@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_kernel_matches_oracle(dtype, case, init):
    Mk, Pk, N, sAD, sX = case
    g = np.random.default_rng(sum(case) + int(init))
    D, A, X = buffers(g, dtype, Mk, Pk, N, sAD, sX, special=True)
    got = run(D, A, X, Mk, Pk, sAD, sX, N, init, dtype)
    ref = oracle.kernel_chain(D, A, X, Mk, Pk, sAD, sX, N, init=init, dtype=dtype)
    same_bits(got, ref)


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_kernel_empty_contraction(dtype):
    g = np.random.default_rng(3)
    D, A, X = buffers(g, dtype, 6, 3, 0, 8, 1)
    same_bits(run(D, A, X, 6, 3, 8, 1, 0, False, dtype), D)                     # D unchanged
    out = run(D, A, X, 6, 3, 8, 1, 0, True, dtype).reshape(3, 8)
    assert np.all(out[:, :6] == 0) and np.array_equal(out[:, 6:], D.reshape(3, 8)[:, 6:])


def test_kernel_tensor_form_and_repeated_accumulation():
    """kernel_ on tensor views sharing one leading dimension; two calls equal the oracle applied
    twice (the chain continues from D's new value)."""
    g = np.random.default_rng(9)
    Mk, Pk, N, ld = 50, 12, 40, 64
    bufD = torch.from_numpy(g.standard_normal((Pk, ld))).cuda()
    bufA = torch.from_numpy(g.standard_normal((N, ld))).cuda()
    Xt = torch.from_numpy(g.standard_normal((Pk, N))).cuda()
    D, A, X = bufD.t()[:Mk, :], bufA.t()[:Mk, :], Xt.t()
    D0 = bufD.cpu().numpy().ravel()
    gbblas.kernel_(D, A, X)
    gbblas.kernel_(D, A, X)
    torch.cuda.synchronize()
    Ah, Xh = bufA.cpu().numpy().ravel(), Xt.cpu().numpy().ravel()
    ref = oracle.kernel_chain(oracle.kernel_chain(D0, Ah, Xh, Mk, Pk, ld, N, N), Ah, Xh, Mk, Pk, ld, N, N)
    same_bits(bufD.cpu().numpy().ravel(), ref)
    gbblas.initkernel_(D, A, X)
    torch.cuda.synchronize()
    same_bits(bufD.cpu().numpy().ravel(), oracle.kernel_chain(ref, Ah, Xh, Mk, Pk, ld, N, N, init=True))
    with pytest.raises(ValueError):
        gbblas.kernel_(D, bufA.t()[:Mk, :].contiguous(), X)     # A's leading dimension differs from D's


def test_kernel_argument_errors():
    L = _lib.lib()
    t = torch.zeros(64, dtype=torch.float64, device="cuda")
    p = ctypes.c_void_p(t.data_ptr())
    st = ctypes.c_void_p(0)
    bad = _lib.GB_ERR_INVALID_VALUE
    assert L.gb_kernel_f64(p, p, p, 4, 2, 3, 4, 4, 0, st) == bad      # stride_AD < Mk
    assert L.gb_kernel_f64(p, p, p, 4, 2, 4, 3, 4, 0, st) == bad      # stride_X < N
    assert L.gb_kernel_f64(p, p, p, 4, 2, 4, 4, 4, 2, st) == bad      # init flag
    assert L.gb_kernel_f64(p, p, p, -1, 2, 4, 4, 4, 0, st) == bad
    host = np.zeros(64)
    assert L.gb_kernel_f64(ctypes.c_void_p(host.ctypes.data), p, p, 4, 2, 4, 4, 4, 0, st) == bad


def test_fastmul_is_jmul_chain():
    """fastmul!(D, A, X) on a small static-size product equals the oracle's jmul! chain bit for bit."""
    g = np.random.default_rng(12)
    A = np.asfortranarray(g.standard_normal((8, 5)))
    X = np.asfortranarray(g.standard_normal((5, 6)))
    D = torch.empty((6, 8), dtype=torch.float64, device="cuda").t()
    gbblas.fastmul_(D, torch.from_numpy(A.T.copy()).cuda().t(), torch.from_numpy(X.T.copy()).cuda().t())
    torch.cuda.synchronize()
    same_bits(np.ascontiguousarray(D.cpu().numpy()), np.ascontiguousarray(oracle.jmul(A, X)))
