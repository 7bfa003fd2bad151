"""The tensor-core tuning table changes how products are scheduled and stored, never their values.

  * digit slices and CRT residues are exact integer sums in FP32, so every engine, band and
    (CRT) number of column panels gives the restatement's bits;
  * FP32 term modes and the adjoint accumulate in the same order whatever the band or the store
    path, so TMA stores of C give the bits of direct stores (ragged shapes included), and a C
    whose layout a TMA map cannot describe (unaligned leading dimension) falls back to direct
    stores;
  * gb_autotune_tc returns a valid tuning, the JSON cache round-trips and installs it.
"""
import json

import numpy as np
import pytest
import torch

import gbblas
from gbblas import tuning, workloads
import oracle
from gpu_util import assert_bit_equal, to_dev, to_dev_ld, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture
def restore_tuning(cuda):
    yield
    for kind in ("ozaki_slices", "ozaki_crt", "f32", "adjoint"):
        for cls in range(3):
            tuning.set_tuning(kind, cls, None)
    gbblas.set_tc_engine(0)


CANDIDATES = [{"engine": 2, "band": 1}, {"engine": 2, "band": 3}, {"engine": 2, "band": 64},
              {"engine": 1, "band": 1}, {"engine": 1, "band": 5}, {"engine": 1, "band": 64}]


@pytest.mark.parametrize("cand", CANDIDATES, ids=["p1", "p3", "p64", "s1", "s5", "s64"])
def test_slices_bit_exact_under_every_engine_and_band(restore_tuning, cand):
    M, K, N = 700, 300, 1100   # several bands and a ragged last band
    g = np.random.default_rng(5)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-6, 7, (M, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    tuning.set_tuning("ozaki_slices", tuning.size_class(M, N), cand)
    Cd = to_dev(np.zeros((M, N)))
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), mode="ozaki", slices=5)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    assert_bit_equal(to_host(Cd), oracle.ozaki_gemm(A, B, slices=5))


@pytest.mark.parametrize("band", [1, 2, 5, 64])
def test_crt_bit_exact_under_every_band(restore_tuning, band):
    M, K, N = 900, 257, 700
    g = np.random.default_rng(6 + band)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-6, 7, (M, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    tuning.set_tuning("ozaki_crt", tuning.size_class(M, N), {"engine": 2, "band": band})
    Cd = to_dev(np.zeros((M, N)))
    gbblas.gemm_(Cd, to_dev(A), to_dev(B), mode="ozaki_crt", slices=12)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    assert_bit_equal(to_host(Cd), oracle.ozaki_crt_gemm(A, B, moduli=12))


def _crt_raw(A, B_phys, tb, N, C0, alpha, beta, moduli):
    M, K = A.shape
    Ad, Bd, Cd = to_dev(A), to_dev(B_phys), to_dev(C0)
    bound = gbblas.gemm_raw(0, tb, M, N, K, alpha, Ad.data_ptr(), M, Bd.data_ptr(), B_phys.shape[0], beta,
                            Cd.data_ptr(), M, dtype=torch.float64, mode=gbblas.MODE_OZAKI_CRT, slices=moduli,
                            stream=torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    return to_host(Cd), bound


@pytest.mark.parametrize("panels", [1, 2, 3, 4])
@pytest.mark.parametrize("tb", [0, 1], ids=["B_k_contiguous", "B_rows_contiguous"])
def test_crt_bit_exact_under_every_panel_count(restore_tuning, panels, tb):
    """Column panels: the residue products of each panel run on the library's high-priority
    stream while the caller's stream splits the next panel of B and reconstructs the previous
    panel of C.  Every panel count gives the restatement's bits, with B stored k-contiguous or
    rows-contiguous, alpha and beta, and a last panel narrower than the others (1100 columns =
    five 256-column tiles)."""
    M, K, N = 700, 257, 1100
    g = np.random.default_rng(40 + panels + 5 * tb)
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)) * np.ldexp(1.0, g.integers(-6, 7, (M, K))))
    Bl = g.uniform(-1, 1, (K, N)) * np.ldexp(1.0, g.integers(-6, 7, (K, N)))
    C0 = np.asfortranarray(g.uniform(-1, 1, (M, N)))
    tuning.set_tuning("ozaki_crt", tuning.size_class(M, N), {"engine": 2, "band": 8, "panels": panels})
    got, _ = _crt_raw(A, np.asfortranarray(Bl.T if tb else Bl), tb, N, C0, 1.5, 0.5, 13)
    assert_bit_equal(got, oracle.ozaki_crt_gemm(A, Bl, C=C0, alpha=1.5, beta=0.5, moduli=13))


@pytest.mark.parametrize("panels", [2, 3, 4])
def test_crt_wide_panel_partitions_match_one_panel(restore_tuning, panels):
    """8192 x 8192 outputs (short K): three panels are a narrow first and last panel (512 and
    1024 columns) around a wide middle one, two panels and 2 x 2 blocks halves; every partition
    gives the bits of one panel over the whole of C, and a grid of entries across the panel
    boundaries equals the restatement."""
    n, K = 8192, 96
    g = np.random.default_rng(90 + panels)
    A = np.asfortranarray(g.uniform(-1, 1, (n, K)) * np.ldexp(1.0, g.integers(-6, 7, (n, K))))
    B = np.asfortranarray(g.uniform(-1, 1, (K, n)) * np.ldexp(1.0, g.integers(-6, 7, (K, n))))
    C0 = torch.rand((n, n), dtype=torch.float64, device="cuda", generator=torch.Generator("cuda").manual_seed(9)).t()
    Ad, Bd = to_dev(A), to_dev(B)
    cls = tuning.size_class(n, n)
    out = {}
    for p in (1, panels):
        tuning.set_tuning("ozaki_crt", cls, {"engine": 2, "band": 8, "panels": p})
        C = C0.clone(memory_format=torch.preserve_format)
        gbblas.gemm_(C, Ad, Bd, 1.5, 0.5, mode="ozaki_crt", slices=12)
        torch.cuda.synchronize()
        gbblas.check_device_status()
        out[p] = C
    assert torch.equal(out[1], out[panels])
    rows = np.array([0, 1, 255, 256, 4095, 4096, 8190, 8191])
    cols = np.array([0, 511, 512, 513, 4095, 4096, 7167, 7168, 8191])
    got = out[panels][torch.as_tensor(rows, device="cuda")][:, torch.as_tensor(cols, device="cuda")].cpu().numpy()
    c0 = C0[torch.as_tensor(rows, device="cuda")][:, torch.as_tensor(cols, device="cuda")].cpu().numpy()
    ref = oracle.ozaki_crt_gemm(np.asfortranarray(A[rows]), np.asfortranarray(B[:, cols]), C=np.asfortranarray(c0),
                                alpha=1.5, beta=0.5, moduli=12)
    assert_bit_equal(got, ref)


def test_crt_panels_with_automatic_plan(restore_tuning):
    """The automatic plan (moduli chosen on the device) read by every panel's kernels."""
    M, K, N = 512, 300, 1024
    A = np.asfortranarray(workloads.ozaki_matrix(M, K, per="row", stream=71))
    B = np.asfortranarray(workloads.ozaki_matrix(K, N, per="col", stream=72))
    tuning.set_tuning("ozaki_crt", tuning.size_class(M, N), {"engine": 2, "band": 2, "panels": 3})
    got, _ = _crt_raw(A, B, 0, N, np.zeros((M, N)), 1.0, 0.0, 0)
    plan = gbblas.last_ozaki_plan()
    assert_bit_equal(got, oracle.ozaki_crt_gemm(A, B, moduli=plan["slices"], bits=plan["bits"]))


def test_crt_panels_from_concurrent_threads(restore_tuning):
    """Two host threads, each on its own stream, make CRT calls in 3 column panels and 2 x 2
    blocks at once: each call takes its own high-priority lane from the device's pool, and
    every result equals the single-panel one."""
    import threading
    M, K, N = 300, 512, 800
    cls = tuning.size_class(M, N)
    ops = []
    for i in range(4):
        A = to_dev(workloads.ozaki_matrix(M, K, per="row", stream=810 + 2 * i))
        B = to_dev(workloads.ozaki_matrix(K, N, per="col", stream=811 + 2 * i))
        ops.append((A, B))
    tuning.set_tuning("ozaki_crt", cls, {"engine": 2, "band": 8, "panels": 1})
    ref = []
    for A, B in ops:
        C = torch.empty((N, M), dtype=torch.float64, device="cuda").t()
        gbblas.gemm_(C, A, B, mode="ozaki_crt", slices=14)
        ref.append(to_host(C))
    for panels in (3, 4):
        tuning.set_tuning("ozaki_crt", cls, {"engine": 2, "band": 8, "panels": panels})
        results, errors = {}, []

        def worker(t):
            try:
                torch.cuda.set_device(0)
                st = torch.cuda.Stream()
                with torch.cuda.stream(st):
                    outs = []
                    for _ in range(3):
                        for A, B in ops[2 * t:2 * t + 2]:
                            C = torch.empty((N, M), dtype=torch.float64, device="cuda").t()
                            gbblas.gemm_(C, A, B, mode="ozaki_crt", slices=14)
                            outs.append(C)
                    st.synchronize()
                    results[t] = [to_host(o) for o in outs]
            except Exception as e:   # surfaced in the main thread
                errors.append(e)

        th = [threading.Thread(target=worker, args=(t,)) for t in (0, 1)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        assert not errors, errors
        gbblas.check_device_status()
        for t in (0, 1):
            for i, got in enumerate(results[t]):
                assert_bit_equal(got, ref[2 * t + i % 2])


def test_crt_panels_short_wait_limit(restore_tuning):
    """A timed-out wait in the residue products of a panel (on the library's lane) is reported
    by the next status check on the caller's stream, and the next call is right."""
    from gbblas import _lib
    g = np.random.default_rng(23)
    M, K, N = 256, 8192, 768
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    Ad, Bd = to_dev(A), to_dev(B)
    C = torch.zeros((N, M), dtype=torch.float64, device="cuda").t()
    tuning.set_tuning("ozaki_crt", tuning.size_class(M, N), {"engine": 2, "band": 8, "panels": 3})
    gbblas.check_device_status()
    gbblas.set_wait_limit_ns(2000)
    try:
        gbblas.gemm_(C, Ad, Bd, mode="ozaki_crt", slices=16)
        torch.cuda.synchronize()
    finally:
        gbblas.set_wait_limit_ns(0)
    with pytest.raises(gbblas.GBError) as e:
        gbblas.check_device_status()
    assert e.value.status == _lib.GB_ERR_PIPELINE_TIMEOUT
    gbblas.gemm_(C, Ad, Bd, mode="ozaki_crt", slices=16)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    assert_bit_equal(to_host(C), oracle.ozaki_crt_gemm(A, B, moduli=16))


def test_crt_panels_under_stream_capture(restore_tuning):
    """Under stream capture a call keeps to one panel on the capturing stream; replays equal
    the eager call made in 3 panels."""
    M, K, N = 384, 1024, 900
    A = to_dev(workloads.ozaki_matrix(M, K, per="row", stream=820))
    B = to_dev(workloads.ozaki_matrix(K, N, per="col", stream=821))
    tuning.set_tuning("ozaki_crt", tuning.size_class(M, N), {"engine": 2, "band": 8, "panels": 3})
    C_eager = torch.empty((N, M), dtype=torch.float64, device="cuda").t()
    gbblas.gemm_(C_eager, A, B, mode="ozaki_crt")
    torch.cuda.synchronize()
    C_graph = torch.empty((N, M), dtype=torch.float64, device="cuda").t()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        gbblas.gemm_(C_graph, A, B, mode="ozaki_crt")
    graph.replay()
    torch.cuda.synchronize()
    gbblas.check_device_status()
    assert_bit_equal(to_host(C_graph), to_host(C_eager))


SHAPES = [(1, 1, 1), (33, 70, 17), (300, 257, 130), (513, 96, 1000), (1024, 512, 768)]


@pytest.mark.parametrize("mode", ["bf16x3", "bf16x6"])
@pytest.mark.parametrize("shape", SHAPES, ids=["x".join(map(str, s)) for s in SHAPES])
def test_f32_tma_store_equals_direct_stores(restore_tuning, mode, shape):
    M, K, N = shape
    g = np.random.default_rng(M + K + N)
    A, B = to_dev(g.standard_normal((M, K)).astype(np.float32)), to_dev(g.standard_normal((K, N)).astype(np.float32))
    cls = tuning.size_class(M, N)
    out = []
    for tma, band in ((0, 8), (1, 8), (1, 3)):
        tuning.set_tuning("f32", cls, {"engine": 2, "band": band, "tma_store": tma})
        Cd = to_dev(np.full((M, N), np.nan, np.float32))
        gbblas.gemm_(Cd, A, B, 1.25, 0.0, mode=mode)
        torch.cuda.synchronize()
        gbblas.check_device_status()
        out.append(to_host(Cd))
    assert_bit_equal(out[1], out[0])
    assert_bit_equal(out[2], out[0])
    assert not np.isnan(out[0]).any()


def test_f32_tma_store_padding_untouched_and_unaligned_fallback(restore_tuning):
    """C inside a larger buffer: rows between M and ldc keep their contents; ldc = M + 1 (not a
    multiple of 4) cannot be a TMA map and takes the direct stores, with the same bits."""
    M, K, N = 130, 200, 90
    g = np.random.default_rng(12)
    A, B = to_dev(g.standard_normal((M, K)).astype(np.float32)), to_dev(g.standard_normal((K, N)).astype(np.float32))
    tuning.set_tuning("f32", 0, {"engine": 2, "band": 8, "tma_store": 1})
    results = []
    for ld in (M + 6, M + 1):   # ld = 136 (TMA-capable), 131 (not)
        Cd, buf = to_dev_ld(np.zeros((M, N), np.float32), ld, fill=7.0)
        gbblas.gemm_(Cd, A, B, mode="bf16x3")
        torch.cuda.synchronize()
        gbblas.check_device_status()
        assert np.all(to_host(buf)[M:, :N] == 7.0)
        results.append(to_host(Cd))
    assert_bit_equal(results[0], results[1])


def test_adjoint_tma_store_equals_direct_stores(restore_tuning):
    M, N, K = 300, 513, 129
    g = np.random.default_rng(21)
    A = to_dev(g.standard_normal((M, K)).astype(np.float32))
    B = to_dev(g.standard_normal((K, N)).astype(np.float32))
    W = to_dev(g.standard_normal((M, N)).astype(np.float32))
    cls = tuning.size_class(max(M, N, K), max(M, N, K))
    got = []
    for tma in (0, 1):
        tuning.set_tuning("adjoint", cls, {"engine": 2, "band": 8, "tma_store": tma})
        dA = torch.full((K, M), float("nan"), dtype=torch.float32, device="cuda").t()
        dB = torch.full((N, K), float("nan"), dtype=torch.float32, device="cuda").t()
        gbblas.gemm_adjoint_(dA, dB, A, B, W)
        torch.cuda.synchronize()
        gbblas.check_device_status()
        got.append((to_host(dA), to_host(dB)))
    assert_bit_equal(got[1][0], got[0][0])
    assert_bit_equal(got[1][1], got[0][1])


def test_autotune_and_cache_roundtrip(restore_tuning, tmp_path):
    cache = str(tmp_path / "tc_tuning.json")
    t, ms = tuning.autotune("f32", 1024, 1024, 512, reps=1, cache=cache)
    assert t.engine in (1, 2) and 1 <= t.band <= 64 and t.tma_store in (0, 1) and ms > 0
    assert tuning.get_tuning("f32", 0).as_dict() == t.as_dict()   # installed
    with open(cache) as f:
        data = json.load(f)
    assert len(data) == 1 and list(data.values())[0]["tuning"] == t.as_dict()
    tuning.set_tuning("f32", 0, None)
    assert tuning.load_cache(cache) == 1
    assert tuning.get_tuning("f32", 0).as_dict() == t.as_dict()
    t2, _ = tuning.autotune("ozaki_crt", 512, 512, 256, reps=1, cache=cache)
    assert t2.engine == 2
