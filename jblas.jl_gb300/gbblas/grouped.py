"""Grouped GEMM host side: problem tables, autotuned tile configurations, CUDA graphs.

jBLAS multiplies each small matrix with its own call (fastmul!/kernel!,
src/kernels.jl:202-208, 239) and a block size fixed by BLASOptions(m_k, p_k)
(src/blas_options.jl:2-7).  Here a ``GroupedGemm`` holds a device table of many
independent products, runs them in one persistent launch (gb_gemm_grouped_*), and can
capture that launch in a CUDA graph.  ``autotune`` times every tile configuration per
size class on the GPU (gb_autotune_grouped) and caches the choice as JSON keyed by the
device and dtype.
"""
import ctypes
import json
import os

import torch

from . import _lib
from ._lib import check

CLASSES = 6
CONFIGS = 10
AUTO = 31   # GB_GROUPED_AUTO: tile configuration chosen per problem by the library's cost model
CLASS_LIMITS = (16, 32, 64, 128, 256)   # max(m, n) upper bounds of classes 0..4; 5 is larger
CONFIG_TILES = {0: (16, 16), 1: (32, 32), 2: (64, 32), 3: (64, 64), 4: (128, 64), 5: (128, 128),
                6: (32, 64), 7: (64, 128), 8: (128, 32), 9: (32, 128), AUTO: "per problem"}


Problem = _lib.Problem
Tuning = _lib.Tuning


def _fn(name):
    return getattr(_lib.lib(), name)


def size_class(m, n):
    d = max(m, n)
    for c, lim in enumerate(CLASS_LIMITS):
        if d <= lim:
            return c
    return CLASSES - 1


def default_tuning(dtype):
    t = Tuning()
    check(_fn("gb_grouped_default_tuning")(8 if dtype == torch.float64 else 4, ctypes.byref(t)),
          "gb_grouped_default_tuning")
    return t


def _colmajor_ld(X, name):
    if X.dim() != 2 or not X.is_cuda:
        raise ValueError("%s must be a 2-D CUDA tensor" % name)
    r, c = X.shape
    if X.numel() == 0:
        return max(1, r)
    s0, s1 = X.stride()
    if not ((s0 == 1 or r <= 1) and (c <= 1 or s1 >= max(1, r))):
        raise ValueError("%s must be column-major (stride (1, ld))" % name)
    return s1 if c > 1 else max(1, r)


class GroupedGemm:
    """C_i = alpha_i A_i B_i + beta_i C_i for every i, in one launch.

    As, Bs, Cs: sequences of column-major CUDA tensors of one dtype (float32/float64).
    The table and the workspace live on the device, so ``run`` is allocation-free and can
    be captured (``capture`` returns a torch.cuda.CUDAGraph replaying the launch)."""

    def __init__(self, As, Bs, Cs, alpha=1.0, beta=0.0, tuning=None):
        if not (len(As) == len(Bs) == len(Cs)):
            raise ValueError("As, Bs and Cs must have the same length")
        self.count = len(As)
        self.dtype = Cs[0].dtype if self.count else torch.float64
        if self.dtype not in (torch.float32, torch.float64):
            raise TypeError("grouped GEMM computes in float32 or float64")
        alphas = alpha if isinstance(alpha, (list, tuple)) else [alpha] * self.count
        betas = beta if isinstance(beta, (list, tuple)) else [beta] * self.count
        host = (Problem * max(1, self.count))()
        self._keep = (list(As), list(Bs), list(Cs))
        for i, (A, B, C) in enumerate(zip(As, Bs, Cs)):
            if A.dtype != self.dtype or B.dtype != self.dtype or C.dtype != self.dtype:
                raise TypeError("all operands must share one dtype")
            m, k = A.shape
            k2, n = B.shape
            if k2 != k or tuple(C.shape) != (m, n):
                raise ValueError("problem %d: A %s, B %s, C %s do not conform" % (i, tuple(A.shape), tuple(B.shape),
                                                                                 tuple(C.shape)))
            host[i] = Problem(m, n, k, _colmajor_ld(A, "A"), _colmajor_ld(B, "B"), _colmajor_ld(C, "C"),
                              A.data_ptr(), B.data_ptr(), C.data_ptr(), float(alphas[i]), float(betas[i]))
        self.host_table = host
        dev = Cs[0].device if self.count else torch.device("cuda")
        raw = bytes(host)[: ctypes.sizeof(Problem) * self.count]
        self.table = torch.frombuffer(bytearray(raw or b"\0"), dtype=torch.uint8).to(dev)
        ws = _fn("gb_grouped_workspace_size")(self.count)
        self.workspace = torch.empty(max(8, ws), dtype=torch.uint8, device=dev)
        self.ws_bytes = ws
        self.tuning = tuning if tuning is not None else default_tuning(self.dtype)

    def sizes(self):
        return [(p.m, p.n, p.k) for p in self.host_table[: self.count]]

    def flops(self):
        return sum(2.0 * p.m * p.n * p.k for p in self.host_table[: self.count])

    def run(self, stream=None):
        name = "gb_gemm_grouped_f64" if self.dtype == torch.float64 else "gb_gemm_grouped_f32"
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        rc = _fn(name)(ctypes.c_void_p(self.table.data_ptr()), self.count, ctypes.byref(self.tuning),
                       ctypes.c_void_p(self.workspace.data_ptr()), self.ws_bytes, ctypes.c_void_p(st))
        check(rc, name)

    def capture(self):
        """A CUDA graph whose replay runs the whole grouped product."""
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            self.run(s.cuda_stream)          # warm-up outside capture
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        with torch.cuda.graph(g):
            self.run(torch.cuda.current_stream().cuda_stream)
        return g


def autotune(plan, reps=3, cache=None):
    """Fastest tile configuration per size class for `plan`'s problems (measured on the GPU).

    With ``cache`` (a JSON path) results are stored under a key made of the device name,
    dtype and the set of size classes present, and reused when the key matches."""
    key = None
    if cache:
        classes = sorted({size_class(m, n) for m, n, _ in plan.sizes()})
        key = "%s|%s|%s" % (torch.cuda.get_device_name(), str(plan.dtype).replace("torch.", ""),
                            ",".join(map(str, classes)))
        if os.path.exists(cache):
            try:
                with open(cache) as f:
                    data = json.load(f)
                if key in data:
                    return Tuning.from_list(data[key]["config"]), data[key].get("class_ms")
            except (OSError, ValueError):
                pass
    out = Tuning()
    ms = (ctypes.c_float * CLASSES)()
    rc = _fn("gb_autotune_grouped")(8 if plan.dtype == torch.float64 else 4, plan.host_table, plan.count,
                                    int(reps), ctypes.byref(out), ms,
                                    ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    check(rc, "gb_autotune_grouped")
    class_ms = [float(x) for x in ms]
    if cache:
        data = {}
        if os.path.exists(cache):
            try:
                with open(cache) as f:
                    data = json.load(f)
            except (OSError, ValueError):
                data = {}
        data[key] = {"config": out.as_list(), "class_ms": class_ms,
                     "tiles": [CONFIG_TILES[c] for c in out.as_list()]}
        os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
        with open(cache, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
    return out, class_ms
