"""gbblas: GB300 (sm_103a) GEMM behind jBLAS.jl's jmul!/gemm! interface.

Everything here calls the C ABI of libgbblas.so (include/gbblas.h); there is no CPU or
PyTorch fallback for any computation.
"""
from . import grouped, tuning
from ._lib import GBError, LIB_PATH, MODE_NATIVE, MODE_OZAKI_BF16, MODE_OZAKI_INT8, MODE_OZAKI_CRT, MODE_BF16X3, MODE_BF16X6, lib
from .api import (DimensionMismatch, GemmFunction, check_device_status, gemm, gemm_, gemm_adjoint_,
                  fastmul_, gemm_autograd, gemm_host, gemm_raw, gemm_semiring, gemm_semiring_, gemm_strided_batched_, initkernel_, jmul_, jmul_host,
                  kernel_, kernel_raw,
                  last_ozaki_plan, launch_counts, ozaki_crt_plan, crt_blocks, ozaki_plan, profile, set_ozaki_min_chunks, set_ozaki_tolerance, set_tc_engine, measure_fma_peaks, set_wait_limit_ns)

__all__ = ["grouped", "tuning", "GBError", "DimensionMismatch", "LIB_PATH", "MODE_NATIVE", "MODE_OZAKI_BF16",
           "MODE_OZAKI_INT8", "MODE_OZAKI_CRT", "MODE_BF16X3", "MODE_BF16X6", "lib", "gemm", "gemm_", "gemm_raw", "gemm_strided_batched_", "gemm_semiring", "gemm_semiring_", "jmul_", "jmul_host", "gemm_host", "fastmul_", "kernel_", "initkernel_", "kernel_raw", "ozaki_plan", "ozaki_crt_plan", "crt_blocks",
           "set_ozaki_tolerance", "set_ozaki_min_chunks", "set_tc_engine", "measure_fma_peaks", "set_wait_limit_ns", "check_device_status", "launch_counts", "last_ozaki_plan",
           "profile", "gemm_adjoint_", "GemmFunction", "gemm_autograd"]
