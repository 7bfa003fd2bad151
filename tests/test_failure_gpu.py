"""Failure detection on the GPU without a fault: bounded pipeline waits.

Every mbarrier wait of the tensor-core kernel has a deadline (gb_set_wait_limit_ns).
Here the deadline is set far below the time one accumulation group takes, so the
epilogue's wait for a finished accumulator runs out: the CTA must record
GB_ERR_PIPELINE_TIMEOUT in the device status word, let its in-flight copies and MMAs
finish, free TMEM and exit.  The host reads the status, the context stays usable and the
next call with the normal limit is correct again.
"""
import numpy as np
import pytest
import torch

import gbblas
from gbblas import _lib
import oracle
from gpu_util import assert_bit_equal, to_dev, to_host

pytestmark = pytest.mark.gpu


def test_short_wait_limit_reports_timeout_and_context_survives(cuda):
    g = np.random.default_rng(21)
    M, K, N = 256, 8192, 512
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    Ad, Bd = to_dev(A), to_dev(B)
    C = torch.zeros((N, M), dtype=torch.float64, device="cuda").t()
    gbblas.check_device_status()                 # start from a clean status word
    gbblas.set_wait_limit_ns(2000)               # 2 us: one group of K = 8192 takes far longer
    try:
        gbblas.gemm_(C, Ad, Bd, mode="ozaki", slices=4)
        torch.cuda.synchronize()                 # the kernel exits instead of hanging
    finally:
        gbblas.set_wait_limit_ns(0)
    with pytest.raises(gbblas.GBError) as e:
        gbblas.check_device_status()
    assert e.value.status == _lib.GB_ERR_PIPELINE_TIMEOUT
    gbblas.check_device_status()                 # reading cleared it
    # the context is still usable and results are right again
    gbblas.gemm_(C, Ad, Bd, mode="ozaki", slices=4)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    assert_bit_equal(to_host(C), oracle.ozaki_gemm(A, B, slices=4))


def test_short_wait_limit_crt_mode(cuda):
    """The same bounded waits guard the residue products of the CRT mode (planner, split and
    combine still run, on whatever the aborted kernel left; the status word says so)."""
    g = np.random.default_rng(22)
    M, K, N = 256, 8192, 512
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    Ad, Bd = to_dev(A), to_dev(B)
    C = torch.zeros((N, M), dtype=torch.float64, device="cuda").t()
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
