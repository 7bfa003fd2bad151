"""The host-buffer entry points (gb_gemm_f64_host / _f32_host / gb_jmul_*_host): the operands live
in host memory as the reference's MMatrix operands do; results equal the oracle (native) and the
device call (Ozaki CRT) bit for bit."""
import ctypes

import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib, workloads
import oracle
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["f64", "f32"])
def test_native_host_matches_oracle(cuda, dtype):
    g = np.random.default_rng(31)
    M, K, N = 130, 77, 95
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)).astype(dtype))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)).astype(dtype))
    C0 = np.asfortranarray(g.uniform(-1, 1, (M, N)).astype(dtype))
    C = C0.copy(order="F")
    gbblas.gemm_host(C, A, B, 1.5, 0.5)
    ref = oracle.gemm(A, B, C=C0, alpha=1.5, beta=0.5, dtype=dtype)
    assert_bit_equal(C, ref)


def test_host_layouts_leading_dimensions_and_transposes(cuda):
    """Row-major operands (read as transposes), strided sub-blocks of larger arrays (lda > rows)
    and a row-major C: every layout gives the same bits; padding outside C is untouched."""
    g = np.random.default_rng(32)
    M, K, N = 70, 45, 33
    A = g.standard_normal((M, K))
    B = g.standard_normal((K, N))
    ref = oracle.gemm(np.asfortranarray(A), np.asfortranarray(B))
    bigA = np.asfortranarray(np.full((M + 9, K + 3), np.nan))
    bigA[:M, :K] = A
    bigC = np.asfortranarray(np.full((M + 5, N + 2), 7.0))
    Cv = bigC[:M, :N]
    gbblas.gemm_host(Cv, bigA[:M, :K], np.ascontiguousarray(B))      # strided A, row-major B
    assert_bit_equal(np.asfortranarray(Cv), ref)
    assert np.all(bigC[M:, :] == 7.0) and np.all(bigC[:, N:] == 7.0)
    Cr = np.zeros((M, N))                                             # row-major C
    gbblas.gemm_host(Cr, np.ascontiguousarray(A), np.asfortranarray(B))
    assert_bit_equal(np.asfortranarray(Cr), ref)


def test_jmul_host(cuda):
    g = np.random.default_rng(33)
    A = np.asfortranarray(g.standard_normal((40, 29)))
    X = np.asfortranarray(g.standard_normal((29, 17)))
    D = np.zeros((40, 17), order="F")
    gbblas.jmul_host(D, A, X)
    assert_bit_equal(D, oracle.jmul(A, X))
    L = _lib.lib()
    Df = np.zeros((40, 17), dtype=np.float32, order="F")
    Af, Xf = A.astype(np.float32, order="F"), X.astype(np.float32, order="F")
    rc = L.gb_jmul_f32_host(ctypes.c_void_p(Df.ctypes.data), ctypes.c_void_p(Af.ctypes.data),
                            ctypes.c_void_p(Xf.ctypes.data), 40, 29, 17, None)
    assert rc == 0
    assert_bit_equal(Df, oracle.jmul(Af, Xf, dtype=np.float32))


def test_crt_host_equals_device_call(cuda):
    M, K, N = 300, 1000, 260
    A = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=81))
    B = np.asfortranarray(workloads.ozaki_matrix(K, N, per="col", stream=82))
    C_host = np.zeros((M, N), order="F")
    _, bound_h = gbblas.gemm_host(C_host, A, B, mode="ozaki_crt", return_bound=True)
    Cd = torch.empty((N, M), dtype=torch.float64, device=cuda).t()
    _, bound_d = gbblas.gemm_(Cd, to_dev(A), to_dev(B), mode="ozaki_crt", return_bound=True)
    assert_bit_equal(C_host, to_host(Cd))
    assert bound_h == bound_d
    assert_bit_equal(C_host, oracle.ozaki_crt_gemm(A, B, moduli=gbblas.last_ozaki_plan()["slices"],
                                                   bits=gbblas.last_ozaki_plan()["bits"]))


@pytest.fixture
def crt_panels(cuda):
    from gbblas import tuning
    yield tuning
    for cls in range(3):
        tuning.set_tuning("ozaki_crt", cls, None)


@pytest.mark.parametrize("panels", [1, 2, 3, 4])
def test_crt_host_pinned_block_copies(crt_panels, panels):
    """Pinned host buffers: a CRT call in blocks copies each block of C to the host C as soon as
    it is reconstructed (column panels, and the quadrants of 2 x 2 blocks into a C with a
    larger leading dimension); the result equals the device call, alpha and beta included, and
    the padding of C is untouched."""
    tuning = crt_panels
    M, K, N = 1100, 300, 2400
    A = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=83))
    B = np.asfortranarray(workloads.ozaki_matrix(K, N, per="col", stream=84))
    C0 = np.asfortranarray(np.random.default_rng(85).uniform(-1, 1, (M, N)))
    tuning.set_tuning("ozaki_crt", tuning.size_class(M, N), {"engine": 2, "band": 8, "panels": panels})
    big = torch.full((N, M + 7), 5.0, dtype=torch.float64).pin_memory()   # column-major, ldc = M + 7
    Ch = big.numpy().T[:M, :]
    Ch[...] = C0
    Ap = torch.from_numpy(np.ascontiguousarray(A.T)).pin_memory().numpy().T
    Bp = torch.from_numpy(np.ascontiguousarray(B.T)).pin_memory().numpy().T
    gbblas.gemm_host(Ch, Ap, Bp, 1.5, 0.5, mode="ozaki_crt", slices=14)
    Cd = to_dev(C0)
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), 1.5, 0.5, mode="ozaki_crt", slices=14)
    assert_bit_equal(np.asfortranarray(Ch), to_host(Cd))
    assert np.all(big.numpy().T[M:, :] == 5.0)


def test_crt_host_pinned_halves_and_narrow_last_panel(crt_panels):
    """8192 x 8192 C (short K) from pinned host buffers in the default three panels: a host call
    cuts them as two halves and a narrow last panel (3584, 3584 and 1024 columns) and copies each
    to the host as it is reconstructed; C equals the device call's over the whole matrix."""
    n, K = 8192, 96
    g = np.random.default_rng(86)
    A = np.asfortranarray(g.uniform(-1, 1, (n, K)) * np.ldexp(1.0, g.integers(-6, 7, (n, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, n)) * np.ldexp(1.0, g.integers(-6, 7, (K, n))))
    pin = lambda X: torch.from_numpy(np.ascontiguousarray(X.T)).pin_memory()   # noqa: E731
    Cp = torch.zeros((n, n), dtype=torch.float64).pin_memory()
    gbblas.gemm_host(Cp.numpy().T, pin(A).numpy().T, pin(B).numpy().T, mode="ozaki_crt", slices=12)
    Cd = torch.empty((n, n), dtype=torch.float64, device="cuda").t()
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), mode="ozaki_crt", slices=12)
    torch.cuda.synchronize()
    assert torch.equal(Cp.t().to("cuda"), Cd)


def test_host_argument_errors(cuda):
    A = np.zeros((4, 4), order="F")
    with pytest.raises(gbblas.GBError):
        L = _lib.lib()
        rc = L.gb_gemm_f64_host(0, 0, 4, 4, 4, 1.0, ctypes.c_void_p(A.ctypes.data), 3, ctypes.c_void_p(A.ctypes.data),
                                4, 0.0, ctypes.c_void_p(A.ctypes.data), 4, 0, 0, None, None)
        _lib.check(rc, "gb_gemm_f64_host")
    with pytest.raises(TypeError):
        gbblas.gemm_host(A, A.astype(np.float32), A)
    with pytest.raises(gbblas.DimensionMismatch):
        gbblas.gemm_host(A, A[:, :3], A)
