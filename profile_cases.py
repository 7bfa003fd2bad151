"""Small single-kernel cases for profiling each gbblas kernel family under ncu.

    python profile_cases.py <case>        (from the repository root, after building the library)

Each case runs one warm-up call and one measured call of the library on seeded inputs
sized for a quick capture (inputs larger than L2 where the kernel streams memory, a few GB
on the device at most), then prints the CUDA-event time of the measured call.

cases:
  native_f64     gb_gemm_f64 NATIVE, 4096^3
  native_f32     gb_gemm_f32, 4096^3
  ozaki          gb_gemm_f64 OZAKI (stats, split, slice products), 4096 x 4096 x 8192
  ozaki_crt      gb_gemm_f64 OZAKI_CRT, 15 moduli (stats, residue split, residue products,
                 CRT combine), 4096 x 4096 x 8192
                 in two column panels (the default tuning at this size)
  ozaki_crt_auto the same with the automatic plan (statistics with the planner's sums)
  ozaki_crt_1panel, ozaki_crt_auto_1panel
                 the same in one panel: every kernel once per call, on the caller's stream
  grouped_f64    gb_gemm_grouped_f64, 4096 problems with m, n, k log-uniform in [8, 512]
  grouped_f32    the same problems in FP32 (default configuration: tiles chosen per problem)
  adjoint        gb_gemm_adjoint_f32, A 4096 x 2048, B 2048 x 4096
  semiring_f32   gb_gemm_semiring_f32 (min, +), 4096^3
  f32_bf16x3     gb_gemm_f32_ex BF16X3 (term split, 3 term products), 4096^3
  f32_bf16x6     gb_gemm_f32_ex BF16X6 (term split, 6 term products), 4096^3
"""
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "jblas.jl_gb300"))
from gbblas import api, grouped, tuning, workloads  # noqa: E402


def _dev_cm(x):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).cuda().t()


def _timed(fn):
    fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def case_native(dtype, n, mode="native"):
    A = (torch.rand((n, n), dtype=dtype, device="cuda") * 2 - 1).t()
    B = (torch.rand((n, n), dtype=dtype, device="cuda") * 2 - 1).t()
    C = torch.empty((n, n), dtype=dtype, device="cuda").t()
    return _timed(lambda: api.gemm_(C, A, B, mode=mode))


def case_ozaki():
    M, N, K = 4096, 4096, 8192
    A = _dev_cm(workloads.ozaki_matrix(M, K, per="row", stream=1))
    B = _dev_cm(workloads.ozaki_matrix(K, N, per="col", stream=2))
    C = torch.empty((N, M), dtype=torch.float64, device="cuda").t()
    return _timed(lambda: api.gemm_(C, A, B, mode="ozaki", slices=10))


def case_ozaki_crt(moduli=15, panels=None):
    """panels: column panels of the call (None = the tuning table's default, 2 at this size;
    1 = every kernel once per call, on the caller's stream)."""
    M, N, K = 4096, 4096, 8192
    A = _dev_cm(workloads.ozaki_matrix(M, K, per="row", stream=1))
    B = _dev_cm(workloads.ozaki_matrix(K, N, per="col", stream=2))
    C = torch.empty((N, M), dtype=torch.float64, device="cuda").t()
    if panels is not None:
        tuning.set_tuning("ozaki_crt", tuning.size_class(M, N), {"engine": 2, "band": 8, "panels": panels})
    return _timed(lambda: api.gemm_(C, A, B, mode="ozaki_crt", slices=moduli))


def case_grouped(dtype=torch.float64, tuning=None):
    sizes = [tuple(int(x) for x in r) for r in workloads.grouped_sizes(4096)]
    As = [(torch.rand((k, m), dtype=dtype, device="cuda") * 2 - 1).t() for m, n, k in sizes]
    Bs = [(torch.rand((n, k), dtype=dtype, device="cuda") * 2 - 1).t() for m, n, k in sizes]
    Cs = [torch.empty((n, m), dtype=dtype, device="cuda").t() for m, n, k in sizes]
    plan = grouped.GroupedGemm(As, Bs, Cs)
    if tuning is not None:
        for i, c in enumerate(tuning):
            plan.tuning.config[i] = c
    return _timed(plan.run)


def case_adjoint():
    M, K, N = 4096, 2048, 4096
    A = _dev_cm(workloads.normal(M, K, stream=51))
    B = _dev_cm(workloads.normal(K, N, stream=52))
    W = _dev_cm(workloads.normal(M, N, stream=53))
    dA = torch.empty((K, M), dtype=torch.float32, device="cuda").t()
    dB = torch.empty((N, K), dtype=torch.float32, device="cuda").t()
    return _timed(lambda: api.gemm_adjoint_(dA, dB, A, B, W))


def case_semiring():
    n = 4096
    A = (torch.rand((n, n), device="cuda") * 200 - 100).t()
    B = (torch.rand((n, n), device="cuda") * 200 - 100).t()
    C = torch.empty((n, n), device="cuda").t()
    return _timed(lambda: api.gemm_semiring_(C, A, B, "min_plus"))


CASES = {
    "native_f64": lambda: case_native(torch.float64, 4096),
    "native_f32": lambda: case_native(torch.float32, 4096),
    "ozaki": case_ozaki,
    "ozaki_crt": case_ozaki_crt,
    "ozaki_crt_auto": lambda: case_ozaki_crt(0),
    "ozaki_crt_1panel": lambda: case_ozaki_crt(15, panels=1),
    "ozaki_crt_auto_1panel": lambda: case_ozaki_crt(0, panels=1),
    "grouped_f64": case_grouped,
    "grouped_f32": lambda: case_grouped(torch.float32),
    "adjoint": case_adjoint,
    "semiring_f32": case_semiring,
    "f32_bf16x3": lambda: case_native(torch.float32, 4096, "bf16x3"),
    "f32_bf16x6": lambda: case_native(torch.float32, 4096, "bf16x6"),
}


def main(argv):
    if len(argv) != 1 or argv[0] not in CASES:
        print(__doc__)
        return 2
    ms = CASES[argv[0]]()
    print("%s: %.3f ms" % (argv[0], ms))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
