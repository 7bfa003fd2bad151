"""Parity at the full benchmark sizes, through sampled entries.

  * plain native GEMM, FP64 and FP32, M = N = K = 8192 and 16384, alpha = 1.5, beta = 0.5,
    uniform[-1, 1) inputs: a 64 x 64 grid of outputs equals jmul!'s FMA chain (the C oracle,
    src/gemm.jl:71-91,149-170) bit for bit;
  * emulated FP64 at 8192^3 on sign * U[1,2) * 2^(e_line + e_elem) inputs:
      - the CRT mode with the plan the library picks: the same grid equals the exact-integer
        restatement of that plan (oracle.ozaki_crt_gemm on the sampled rows of A and columns
        of B: row exponents depend on the whole row only, so the restatement of the sampled
        block is the sampled block of the restatement);
      - the digit-slice sweep s = 3..8 plus the automatic plan, and the moduli sweep
        n = 8..16 plus the automatic plan: each bit-exact on the grid against its restatement,
        its normwise error (binary128 dot products on the grid) below the bound the call
        returns, and the bounds decreasing with s and n.
Inputs for the native cases are drawn on the device (seeded torch generator); only the
sampled rows and columns travel to the host.
"""
import numpy as np
import pytest
import torch

import gbblas
from gbblas import workloads
import oracle
from gpu_util import assert_bit_equal, to_dev

pytestmark = pytest.mark.gpu

GRID = 64


def _grid(M, N, seed):
    g = np.random.default_rng(seed)
    return np.sort(g.choice(M, GRID, replace=False)), np.sort(g.choice(N, GRID, replace=False))


def _pairs():
    ii, jj = np.meshgrid(np.arange(GRID), np.arange(GRID), indexing="ij")
    return ii.ravel(), jj.ravel()


def _block(X, r, c):
    return X[torch.as_tensor(r, device=X.device)][:, torch.as_tensor(c, device=X.device)]


@pytest.mark.parametrize("n", [8192, 16384])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_native_config_sizes_sampled_bit_exact(cuda, dtype, n):
    gen = torch.Generator(device=cuda).manual_seed(n + (64 if dtype == torch.float64 else 32))
    A = (torch.rand((n, n), generator=gen, dtype=dtype, device=cuda) * 2 - 1).t()
    B = (torch.rand((n, n), generator=gen, dtype=dtype, device=cuda) * 2 - 1).t()
    C = (torch.rand((n, n), generator=gen, dtype=dtype, device=cuda) * 2 - 1).t()
    r, c = _grid(n, n, n + 1)
    As = np.asfortranarray(_block(A, r, np.arange(n)).cpu().numpy())
    Bs = np.asfortranarray(_block(B, np.arange(n), c).cpu().numpy())
    Cs = np.asfortranarray(_block(C, r, c).cpu().numpy())
    gbblas.gemm_(C, A, B, 1.5, 0.5)
    torch.cuda.synchronize()
    got = _block(C, r, c).cpu().numpy()
    ii, jj = _pairs()
    npdt = np.float64 if dtype == torch.float64 else np.float32
    ref = oracle.chain_entries(As, Bs, ii, jj, C=Cs, alpha=1.5, beta=0.5, dtype=npdt)
    assert_bit_equal(got[ii, jj], ref)


@pytest.fixture(scope="module")
def ozaki_8192(cuda):
    n = 8192
    A = np.asfortranarray(workloads.ozaki_matrix(n, n, per="row", stream=1))
    B = np.asfortranarray(workloads.ozaki_matrix(n, n, per="col", stream=2))
    r, c = _grid(n, n, 77)
    As = np.asfortranarray(A[r, :])
    Bs = np.asfortranarray(B[:, c])
    ii, jj = _pairs()
    hi, lo = oracle.quad_entries(As, Bs, ii, jj)
    return {"n": n, "Ad": to_dev(A), "Bd": to_dev(B), "r": r, "c": c, "As": As, "Bs": Bs, "hi": hi, "lo": lo,
            "na": float(np.linalg.norm(A)), "nb": float(np.linalg.norm(B))}


def _ozaki_call(w, mode, slices):
    n = w["n"]
    C = torch.empty((n, n), dtype=torch.float64, device=w["Ad"].device).t()
    _, bound = gbblas.gemm_(C, w["Ad"], w["Bd"], mode=mode, slices=slices, return_bound=True)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    plan = gbblas.last_ozaki_plan()
    got = _block(C, w["r"], w["c"]).cpu().numpy()
    ii, jj = _pairs()
    d = (got[ii, jj] - w["hi"]) - w["lo"]
    err = float(np.linalg.norm(d) * np.sqrt(n * n / ii.size) / (w["na"] * w["nb"]))
    return got, bound, plan, err


def test_crt_8192_automatic_plan_sampled_bit_exact(ozaki_8192):
    w = ozaki_8192
    got, bound, plan, err = _ozaki_call(w, "ozaki_crt", 0)
    ref = oracle.ozaki_crt_gemm(w["As"], w["Bs"], moduli=plan["slices"], bits=plan["bits"])
    assert_bit_equal(got, ref)
    assert err <= bound <= 2.0 ** -50


def test_slices_8192_sweep(ozaki_8192):
    """Digit slices s = 3..8 (FP32 accumulation of BF16 digit products) and the automatic s."""
    w = ozaki_8192
    prev = np.inf
    for s in (3, 4, 5, 6, 7, 8, 0):
        got, bound, plan, err = _ozaki_call(w, "ozaki", s)
        if s:
            assert plan["slices"] == s
        ref = oracle.ozaki_gemm(w["As"], w["Bs"], slices=plan["slices"],
                                min_chunks=oracle.chunks_for(w["n"], plan["k_chunk"]))
        assert_bit_equal(got, ref)
        assert err <= bound, (s, err, bound)
        if s:
            assert bound < prev, (s, bound, prev)
            prev = bound
        else:
            assert bound <= 2.0 ** -50


def test_crt_8192_moduli_sweep(ozaki_8192):
    """Moduli n = 8..16 (one BF16 residue product each, exact FP32 sums) and the automatic n."""
    w = ozaki_8192
    prev = np.inf
    for m in (8, 9, 10, 11, 12, 13, 14, 15, 16, 0):
        got, bound, plan, err = _ozaki_call(w, "ozaki_crt", m)
        if m:
            assert plan["slices"] == m and plan["bits"] == oracle.crt_bits_for(w["n"], m)
        ref = oracle.ozaki_crt_gemm(w["As"], w["Bs"], moduli=plan["slices"], bits=plan["bits"])
        assert_bit_equal(got, ref)
        assert err <= bound, (m, err, bound)
        if m:
            assert bound < prev, (m, bound, prev)
            prev = bound
        else:
            assert bound <= 2.0 ** -50


@pytest.mark.parametrize("panels", [1, 2])
@pytest.mark.parametrize("mode", ["ozaki_crt", "ozaki"])
def test_k_contiguous_operand_beyond_65535_rows(cuda, mode, panels):
    """B with 66000 columns stored k-contiguous: its digit or residue planes are written by row
    bands of at most 65535 rows (the grid's y limit), all into the planes of the whole operand.
    Columns on both sides of every band edge and of the CRT panel edge match the restatement
    bit for bit."""
    from gbblas import tuning
    M, K, N = 64, 64, 66000
    g = np.random.default_rng(123 + panels)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-6, 7, (M, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-6, 7, (K, N))))
    cls = tuning.size_class(M, N)
    try:
        if mode == "ozaki_crt":
            tuning.set_tuning("ozaki_crt", cls, {"engine": 2, "band": 8, "panels": panels})
        elif panels > 1:
            pytest.skip("column panels are a CRT option")
        Cd = to_dev(np.zeros((M, N)))
        gbblas.gemm_(Cd, to_dev(A), to_dev(B), mode=mode, slices=12 if mode == "ozaki_crt" else 5)
        torch.cuda.synchronize()
        gbblas.check_device_status()
    finally:
        tuning.set_tuning("ozaki_crt", cls, None)
    edges = [0, 1, 32767, 32768, 33023, 33024, 65534, 65535, 65536, 65999]
    cols = np.unique(np.concatenate([edges, g.choice(N, 22, replace=False)]))
    got = Cd[:, torch.from_numpy(cols).to(Cd.device)].cpu().numpy()
    Bs = np.asfortranarray(B[:, cols])
    ref = (oracle.ozaki_crt_gemm(A, Bs, moduli=12) if mode == "ozaki_crt" else oracle.ozaki_gemm(A, Bs, slices=5))
    assert_bit_equal(np.asfortranarray(got), ref)
