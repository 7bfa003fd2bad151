"""GPU checks of the grouped (batched, uneven) GEMM: one persistent launch, many problems.

Every tile configuration computes jmul!'s per-element FMA chain in the reference's K
order, so every check is bit-exact against the oracle, whatever the tuning."""
import ctypes

import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib, grouped, workloads
import oracle
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu


def make_problems(sizes, dtype, seed, alpha=1.0, beta=0.0):
    g = np.random.default_rng(seed)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    hA, hB, hC, As, Bs, Cs = [], [], [], [], [], []
    for m, n, k in sizes:
        A = np.asfortranarray(g.uniform(-1, 1, (m, k)).astype(npdt))
        B = np.asfortranarray(g.uniform(-1, 1, (k, n)).astype(npdt))
        C = np.asfortranarray(g.uniform(-1, 1, (m, n)).astype(npdt))
        hA.append(A); hB.append(B); hC.append(C)
        As.append(to_dev(A)); Bs.append(to_dev(B)); Cs.append(to_dev(C))
    return hA, hB, hC, As, Bs, Cs


def check_all(hA, hB, hC, Cs, dtype, alphas, betas):
    npdt = np.float64 if dtype == torch.float64 else np.float32
    torch.cuda.synchronize()
    for A, B, C0, Cd, a, b in zip(hA, hB, hC, Cs, alphas, betas):
        ref = oracle.gemm(A, B, C=C0, alpha=a, beta=b, dtype=npdt)
        assert_bit_equal(to_host(Cd), ref)


SIZES = [(1, 1, 1), (7, 5, 3), (16, 16, 16), (17, 33, 9), (64, 64, 64), (65, 31, 130), (129, 257, 70),
         (300, 20, 257), (8, 512, 40), (513, 9, 11), (200, 200, 0)]


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_bit_exact_default_tuning(cuda, dtype):
    hA, hB, hC, As, Bs, Cs = make_problems(SIZES, dtype, 1)
    alphas = [1.0, 1.5, -2.0, 0.0, 1.0, 0.5, 1.0, 2.0, 1.0, 1.0, 1.0]
    betas = [0.0, 0.5, 1.0, 0.5, 0.0, 0.0, 1.0, 0.25, 0.0, 0.5, 0.5]
    plan = grouped.GroupedGemm(As, Bs, Cs, alpha=alphas, beta=betas)
    plan.run()
    check_all(hA, hB, hC, Cs, dtype, alphas, betas)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_every_configuration_bit_exact(cuda, dtype):
    """Every tile configuration (and the per-problem choice) gives jmul!'s chain bit for bit,
    with alpha/beta (including alpha = 0: C = beta C without reading A and B)."""
    g = np.random.default_rng(2)
    sizes = [tuple(int(x) for x in g.integers(1, 300, 3)) for _ in range(24)] + [(300, 5, 40), (5, 300, 40)]
    nconf = 4 if dtype == torch.float64 else grouped.CONFIGS
    alphas = [1.0] * (len(sizes) - 2) + [0.0, 1.5]
    betas = [0.0] * (len(sizes) - 3) + [0.5, 0.5, -0.25]
    for cfg in list(range(nconf)) + [grouped.AUTO]:
        hA, hB, hC, As, Bs, Cs = make_problems(sizes, dtype, 3 + (cfg % 16))
        plan = grouped.GroupedGemm(As, Bs, Cs, alpha=alphas, beta=betas,
                                   tuning=grouped.Tuning.from_list([cfg] * grouped.CLASSES))
        plan.run()
        check_all(hA, hB, hC, Cs, dtype, alphas, betas)


def test_invalid_tuning_rejected(cuda):
    hA, hB, hC, As, Bs, Cs = make_problems([(8, 8, 8)], torch.float64, 4)
    plan = grouped.GroupedGemm(As, Bs, Cs, tuning=grouped.Tuning.from_list([5] * grouped.CLASSES))
    with pytest.raises(gbblas.GBError) as e:     # configurations 4 to 9 are float32 only
        plan.run()
    assert e.value.status == _lib.GB_ERR_INVALID_VALUE


def test_cuda_graph_replay(cuda):
    sizes = [tuple(int(x) for x in row) for row in workloads.grouped_sizes(256, seed=5)]
    hA, hB, hC, As, Bs, Cs = make_problems(sizes, torch.float64, 6)
    plan = grouped.GroupedGemm(As, Bs, Cs, alpha=1.0, beta=0.0)
    graph = plan.capture()
    for C in Cs:
        C.fill_(float("nan"))
    graph.replay()
    check_all(hA, hB, hC, Cs, torch.float64, [1.0] * len(sizes), [0.0] * len(sizes))


def test_autotune_and_cache(cuda, tmp_path):
    sizes = [tuple(int(x) for x in row) for row in workloads.grouped_sizes(300, seed=7)]
    hA, hB, hC, As, Bs, Cs = make_problems(sizes, torch.float32, 8)
    plan = grouped.GroupedGemm(As, Bs, Cs, beta=0.5)
    before = [to_host(C) for C in Cs]
    cache = str(tmp_path / "tune.json")
    tuning, ms = grouped.autotune(plan, reps=2, cache=cache)
    # FP32: any of the tile configurations or the per-problem choice
    assert all(0 <= c < grouped.CONFIGS or c == grouped.AUTO for c in tuning.as_list())
    for C, b in zip(Cs, before):                 # tuning leaves the caller's C untouched
        assert np.array_equal(to_host(C), b)
    again, _ = grouped.autotune(plan, reps=2, cache=cache)
    assert again.as_list() == tuning.as_list()
    plan.tuning = tuning
    plan.run()
    check_all(hA, hB, hC, Cs, torch.float32, [1.0] * len(sizes), [0.5] * len(sizes))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_grouped_4096_loguniform_problems(cuda, dtype):
    """4096 problems, m, n, k log-uniform in [8, 512]; 128 sampled problems vs the oracle."""
    sizes = [tuple(int(x) for x in row) for row in workloads.grouped_sizes(4096)]
    g = np.random.default_rng(9)
    npdt = np.float64 if dtype == torch.float64 else np.float32
    As, Bs, Cs = [], [], []
    for m, n, k in sizes:
        As.append(torch.rand((k, m), dtype=dtype, device="cuda").t() * 2 - 1)
        Bs.append(torch.rand((n, k), dtype=dtype, device="cuda").t() * 2 - 1)
        Cs.append(torch.empty((n, m), dtype=dtype, device="cuda").t())
    As = [a.t().contiguous().t() for a in As]
    Bs = [b.t().contiguous().t() for b in Bs]
    plan = grouped.GroupedGemm(As, Bs, Cs)
    plan.run()
    torch.cuda.synchronize()
    for i in g.choice(len(sizes), 128, replace=False):
        ref = oracle.gemm(to_host(As[i]), to_host(Bs[i]), dtype=npdt)
        assert_bit_equal(to_host(Cs[i]), ref)
