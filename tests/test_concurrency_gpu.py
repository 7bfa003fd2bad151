"""Concurrent use of the library: several streams and host threads at once.

Every call is stream-ordered and keeps its state (workspace, CRT plan record) to itself, so
interleaved calls on different streams, from different threads, give the same bits as the
same calls made one after another; each thread's gb_last_ozaki_plan reports its own last call.
"""
import threading

import numpy as np
import pytest
import torch

import gbblas
from gbblas import workloads
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu


def problems(n, seed0):
    out = []
    for i in range(n):
        M, K, N = 96 + 32 * i, 256 + 64 * i, 80 + 16 * i
        A = to_dev(workloads.ozaki_matrix(M, K, per="row", stream=seed0 + 2 * i))
        B = to_dev(workloads.ozaki_matrix(K, N, per="col", stream=seed0 + 2 * i + 1))
        out.append((A, B))
    return out


def call(A, B, mode, slices):
    C = torch.empty((B.shape[1], A.shape[0]), dtype=torch.float64, device=A.device).t()
    gbblas.gemm_(C, A, B, mode=mode, slices=slices)
    return C


CALLS = [("ozaki_crt", 0), ("ozaki_crt", 14), ("native", 0), ("ozaki_crt", 20), ("ozaki_crt", 0), ("native", 0)]


def test_interleaved_streams_bit_exact(cuda):
    probs = problems(len(CALLS), 400)
    ref = []
    for (A, B), (mode, sl) in zip(probs, CALLS):
        ref.append(to_host(call(A, B, mode, sl)))
    torch.cuda.synchronize()
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    outs = []
    for i, ((A, B), (mode, sl)) in enumerate(zip(probs, CALLS)):
        st = streams[i % 2]
        st.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(st):
            outs.append(call(A, B, mode, sl))
    torch.cuda.synchronize()
    gbblas.check_device_status()
    for got, want in zip(outs, ref):
        assert_bit_equal(to_host(got), want)


def test_threads_bit_exact_and_own_last_plan(cuda):
    probs = {0: problems(4, 500), 1: problems(4, 600)}
    moduli = {0: 13, 1: 17}
    ref = {t: [to_host(call(A, B, "ozaki_crt", moduli[t])) for A, B in probs[t]] for t in (0, 1)}
    torch.cuda.synchronize()
    results, plans, errors = {}, {}, []

    def worker(t):
        try:
            torch.cuda.set_device(0)
            st = torch.cuda.Stream()
            with torch.cuda.stream(st):
                outs = []
                for _ in range(3):
                    for A, B in probs[t]:
                        outs.append(call(A, B, "ozaki_crt", moduli[t]))
                        gbblas.gemm_(torch.empty_like(outs[-1].t()).t(), A, B, mode="native")
                st.synchronize()
                plans[t] = gbblas.last_ozaki_plan()
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
            assert_bit_equal(got, ref[t][i % len(probs[t])])
        assert plans[t]["slices"] == moduli[t]


def test_plan_readback_reports_reuse_instead_of_another_calls_plan(cuda):
    """After as many later CRT calls on the device as the read-back ring holds, this thread's
    last plan is reported as unavailable rather than replaced by another call's plan."""
    A = to_dev(workloads.ozaki_matrix(64, 64, per="row", stream=700))
    B = to_dev(workloads.ozaki_matrix(64, 64, per="col", stream=701))
    call(A, B, "ozaki_crt", 7)
    torch.cuda.synchronize()

    def flood():
        torch.cuda.set_device(0)
        C = torch.empty((64, 64), dtype=torch.float64, device="cuda").t()
        for _ in range(4096):
            gbblas.gemm_(C, A, B, mode="ozaki_crt", slices=9)
        torch.cuda.synchronize()
        assert gbblas.last_ozaki_plan()["slices"] == 9          # that thread's own last call

    th = threading.Thread(target=flood)
    th.start()
    th.join()
    with pytest.raises(gbblas.GBError):
        gbblas.last_ozaki_plan()
    call(A, B, "ozaki_crt", 7)
    assert gbblas.last_ozaki_plan()["slices"] == 7
