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


def test_short_wait_limit_adjoint(cuda):
    """The fused adjoint runs on the same pipeline: an expired wait is reported through the
    status word and the next call is within its tolerance again."""
    g = np.random.default_rng(23)
    M, K, N = 512, 4096, 512
    A = torch.from_numpy(g.standard_normal((K, M)).astype(np.float32)).cuda().t()
    B = torch.from_numpy(g.standard_normal((N, K)).astype(np.float32)).cuda().t()
    W = torch.from_numpy(g.standard_normal((N, M)).astype(np.float32)).cuda().t()
    dA = torch.empty((K, M), dtype=torch.float32, device="cuda").t()
    dB = torch.empty((N, K), dtype=torch.float32, device="cuda").t()
    gbblas.check_device_status()
    gbblas.set_wait_limit_ns(2000)
    try:
        gbblas.gemm_adjoint_(dA, dB, A, B, W)
        torch.cuda.synchronize()
    finally:
        gbblas.set_wait_limit_ns(0)
    with pytest.raises(gbblas.GBError) as e:
        gbblas.check_device_status()
    assert e.value.status == _lib.GB_ERR_PIPELINE_TIMEOUT
    gbblas.gemm_adjoint_(dA, dB, A, B, W)
    torch.cuda.synchronize()
    gbblas.check_device_status()
    ref = (W.double() @ B.double().t()).cpu().numpy()
    bound = (2.0 ** -15 + N * 2.0 ** -24) * (W.double().abs() @ B.double().abs().t()).cpu().numpy()
    assert np.all(np.abs(dA.double().cpu().numpy() - ref) <= bound + 1e-30)


def test_short_wait_limit_host_buffer_call(cuda):
    """The blocking host-buffer call returns the expired wait as its own status (it reads and
    clears the status word), and the next call is right."""
    g = np.random.default_rng(24)
    M, K, N = 256, 8192, 256
    A = np.asfortranarray(g.uniform(-1, 1, (M, K)))
    B = np.asfortranarray(g.uniform(-1, 1, (K, N)))
    C = np.zeros((M, N), order="F")
    gbblas.check_device_status()
    gbblas.set_wait_limit_ns(2000)
    try:
        with pytest.raises(gbblas.GBError) as e:
            gbblas.gemm_host(C, A, B, mode="ozaki_crt", slices=16)
    finally:
        gbblas.set_wait_limit_ns(0)
    assert e.value.status == _lib.GB_ERR_PIPELINE_TIMEOUT
    gbblas.check_device_status()                      # cleared by the call itself
    gbblas.gemm_host(C, A, B, mode="ozaki_crt", slices=16)
    assert_bit_equal(C, oracle.ozaki_crt_gemm(A, B, moduli=16))
