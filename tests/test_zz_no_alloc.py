"""The allocation-free grouped FP64 entry point (gb_gemm_grouped_f64_noalloc).

Some callers cannot allocate device memory at the moment they multiply: threads that
must not stall on the device synchronisation cudaMalloc/cudaFree can imply, and hosts
whose device memory is owned by another runtime.  This entry point keeps its scratch (the
per-problem tile prefix sums) in a fixed device array of GB_GROUPED_NOALLOC_MAX + 1
entries.  The test calls it through the C ABI, twice in a row on different problem sets
(the second call must not see the first call's leftover contents), and compares each
result with the regular gb_gemm_grouped_f64 entry point, bit for bit as every grouped
test does.  It is collected last and also runs alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib, grouped, workloads
from gpu_util import assert_bit_equal, to_host

pytestmark = pytest.mark.gpu


def _problem_set(count, seed):
    sizes = [tuple(int(x) for x in row) for row in workloads.grouped_sizes(count, lo=1, hi=300, seed=seed)]
    g = torch.Generator(device="cuda").manual_seed(seed)
    As, Bs, Cs, Rs = [], [], [], []
    for m, n, k in sizes:
        As.append((torch.rand((k, m), generator=g, dtype=torch.float64, device="cuda") * 2 - 1).t())
        Bs.append((torch.rand((n, k), generator=g, dtype=torch.float64, device="cuda") * 2 - 1).t())
        c0 = (torch.rand((n, m), generator=g, dtype=torch.float64, device="cuda") * 2 - 1).t()
        Cs.append(c0.t().contiguous().t())
        Rs.append(c0.t().contiguous().t())
    return As, Bs, Cs, Rs


def _noalloc(plan, stream):
    rc = _lib.lib().gb_gemm_grouped_f64_noalloc(ctypes.c_void_p(plan.table.data_ptr()), plan.count,
                                                ctypes.byref(plan.tuning), ctypes.c_void_p(stream))
    _lib.check(rc, "gb_gemm_grouped_f64_noalloc")


@pytest.mark.parametrize("first,second", [(700, 180)])
def test_noalloc_matches_grouped_two_calls(cuda, first, second):
    stream = torch.cuda.current_stream().cuda_stream
    for count, seed, beta in ((first, 11, 0.5), (second, 12, 0.0)):
        As, Bs, Cs, Rs = _problem_set(count, seed)
        ref_plan = grouped.GroupedGemm(As, Bs, Rs, alpha=1.25, beta=beta)
        plan = grouped.GroupedGemm(As, Bs, Cs, alpha=1.25, beta=beta)
        ref_plan.run(stream)            # the regular entry point (workspace from the caller)
        _noalloc(plan, stream)
        torch.cuda.synchronize()
        for C, R in zip(Cs, Rs):
            assert_bit_equal(to_host(C), to_host(R))


def test_noalloc_rejects_oversized_count(cuda):
    dummy = torch.zeros(ctypes.sizeof(_lib.Problem), dtype=torch.uint8, device="cuda")
    rc = _lib.lib().gb_gemm_grouped_f64_noalloc(ctypes.c_void_p(dummy.data_ptr()), 65537, None,
                                                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == _lib.GB_ERR_INVALID_VALUE
    torch.cuda.synchronize()


def test_noalloc_rejects_null_and_host_tables(cuda):
    """A null table or a table in host memory is refused with GB_ERR_INVALID_VALUE before any
    launch (a kernel given either would fault), and the next call still works."""
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    L = _lib.lib()
    host_table = (_lib.Problem * 4)()
    assert L.gb_gemm_grouped_f64_noalloc(None, 4, None, stream) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_gemm_grouped_f64_noalloc(ctypes.cast(host_table, ctypes.c_void_p), 4, None,
                                         stream) == _lib.GB_ERR_INVALID_VALUE
    assert L.gb_gemm_grouped_f64_noalloc(None, 0, None, stream) == _lib.GB_OK
    torch.cuda.synchronize()
    As, Bs, Cs, Rs = _problem_set(40, 13)
    ref_plan = grouped.GroupedGemm(As, Bs, Rs)
    plan = grouped.GroupedGemm(As, Bs, Cs)
    ref_plan.run(stream.value)
    _noalloc(plan, stream.value)
    torch.cuda.synchronize()
    for C, R in zip(Cs, Rs):
        assert_bit_equal(to_host(C), to_host(R))
