"""Host-side mirror of jBLAS's matrix-multiply interface over the gbblas C ABI.

Reference interface (paths relative to the jBLAS.jl tree):
  jmul!(D, A, X)  src/gemm.jl:244-348   D (M x P) = A (M x N) * X (N x P), returns D
  kernel!(pD, pA, pX, Kernel{...})       src/kernels.jl:239 (pointer form, D += A*X)

``jmul_`` keeps jmul!'s argument order, meaning (the reference's N is the contraction
dimension) and in-place contract: D is overwritten and returned.  ``gemm_`` is the
BLAS-3 generalisation (alpha, beta, transposes, FP64 mode).  Matrices are CUDA torch
tensors; column-major storage (stride (1, ld)) is used as is, row-major storage is
read as the transpose of a column-major matrix, so no copy is made for either.
Shape errors raise ``DimensionMismatch`` (jmul!'s sizes are type parameters, so the
reference reports them as a method error at compile time); library errors raise
``GBError`` with the status string.
"""
import ctypes

import torch

from . import _lib
from ._lib import GBError, check


class DimensionMismatch(ValueError):
    """Operand shapes do not conform (Julia's DimensionMismatch)."""


def _stream_ptr(t):
    return ctypes.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


def _storage(X, name, allow_copy):
    """(tensor, ld, trans) with X == (trans ? S^T : S) for column-major S of leading dim ld."""
    if X.dim() != 2:
        raise DimensionMismatch("%s must be a matrix, got %d dims" % (name, X.dim()))
    if not X.is_cuda:
        raise ValueError("%s must be a CUDA tensor (device memory)" % name)
    r, c = X.shape
    s0, s1 = X.stride()
    if (s0 == 1 or r <= 1) and (c <= 1 or s1 >= max(1, r)):
        return X, (s1 if c > 1 else max(1, r)), 0
    if (s1 == 1 or c <= 1) and (r <= 1 or s0 >= max(1, c)):
        return X, (s0 if r > 1 else max(1, c)), 1
    if not allow_copy:
        raise ValueError("%s must have unit stride in one dimension" % name)
    Y = X.t().contiguous().t()
    return Y, max(1, r), 0


def _dtype_of(*ts):
    dt = ts[0].dtype
    for t in ts[1:]:
        if t.dtype != dt:
            raise TypeError("all operands must share one dtype, got %s and %s" % (dt, t.dtype))
    if dt not in (torch.float64, torch.float32):
        raise TypeError("gbblas computes in float64 or float32, got %s" % dt)
    return dt


def gemm_raw(transA, transB, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, *, dtype,
             mode=_lib.MODE_NATIVE, slices=0, want_bound=False, stream=None):
    """Direct C-ABI call on device pointers (ints).  Returns the error bound or None."""
    L = _lib.lib()
    st = ctypes.c_void_p(stream)
    if dtype == torch.float64:
        bound = ctypes.c_double(0.0)
        rc = L.gb_gemm_f64(int(transA), int(transB), M, N, K, float(alpha), ctypes.c_void_p(A), lda,
                           ctypes.c_void_p(B), ldb, float(beta), ctypes.c_void_p(C), ldc, int(mode),
                           int(slices), ctypes.byref(bound) if want_bound else None, st)
        check(rc, "gb_gemm_f64")
        return bound.value if want_bound else None
    if mode in (_lib.MODE_OZAKI_BF16, _lib.MODE_OZAKI_INT8, _lib.MODE_OZAKI_CRT):
        raise ValueError("Ozaki modes emulate float64; float32 runs natively or in a BF16 term mode")
    if mode == _lib.MODE_NATIVE:
        rc = L.gb_gemm_f32(int(transA), int(transB), M, N, K, float(alpha), ctypes.c_void_p(A), lda,
                           ctypes.c_void_p(B), ldb, float(beta), ctypes.c_void_p(C), ldc, st)
        check(rc, "gb_gemm_f32")
    else:
        rc = L.gb_gemm_f32_ex(int(transA), int(transB), M, N, K, float(alpha), ctypes.c_void_p(A), lda,
                              ctypes.c_void_p(B), ldb, float(beta), ctypes.c_void_p(C), ldc, int(mode), st)
        check(rc, "gb_gemm_f32_ex")
    return None


_MODES = {"native": _lib.MODE_NATIVE, "ozaki": _lib.MODE_OZAKI_BF16,
          "ozaki_bf16": _lib.MODE_OZAKI_BF16, "ozaki_int8": _lib.MODE_OZAKI_INT8,
          "ozaki_crt": _lib.MODE_OZAKI_CRT, "bf16x3": _lib.MODE_BF16X3, "bf16x6": _lib.MODE_BF16X6}


def gemm_(C, A, B, alpha=1.0, beta=0.0, *, mode="native", slices=0, return_bound=False):
    """C = alpha * A @ B + beta * C in place; A (M x K), B (K x N), C (M x N).

    mode "native": the jmul! FMA chain (bit-identical to the oracle); "bf16x3" / "bf16x6"
    (float32 only): BF16 term products on the tensor cores (2 terms, 3 products / 3 terms, 6
    products; componentwise error about (2^-15 / 2^-21 + K 2^-24) |A||B|); "ozaki": FP64
    emulation on BF16 tensor cores by digit slices (float64 only; slices = 0 picks the
    count for the library tolerance); "ozaki_crt": FP64 emulation by residue products
    and the Chinese remainder theorem (slices = number of moduli, 0 = automatic).  With return_bound the a-priori normwise error bound is
    returned alongside C.
    """
    dt = _dtype_of(C, A, B)
    M, K = A.shape
    K2, N = B.shape
    if K2 != K or tuple(C.shape) != (M, N):
        raise DimensionMismatch("A is %dx%d, B is %dx%d, C is %dx%d" % (M, K, K2, N, *C.shape))
    md = _MODES[mode] if isinstance(mode, str) else int(mode)
    Cs, ldc, tc = _storage(C, "C", allow_copy=False)
    As, lda, ta = _storage(A, "A", allow_copy=True)
    Bs, ldb, tb = _storage(B, "B", allow_copy=True)
    stream = torch.cuda.current_stream(C.device).cuda_stream
    if tc == 0:
        bound = gemm_raw(ta, tb, M, N, K, alpha, As.data_ptr(), lda, Bs.data_ptr(), ldb, beta,
                         Cs.data_ptr(), ldc, dtype=dt, mode=md, slices=slices,
                         want_bound=return_bound, stream=stream)
    else:
        # C stored row-major: C^T (N x M, column-major) = B^T A^T
        bound = gemm_raw(1 - tb, 1 - ta, N, M, K, alpha, Bs.data_ptr(), ldb, As.data_ptr(), lda,
                         beta, Cs.data_ptr(), ldc, dtype=dt, mode=md, slices=slices,
                         want_bound=return_bound, stream=stream)
    return (C, bound) if return_bound else C


def _host_storage(X, name, out=False):
    """(array, ld, trans) for a 2-D numpy array with a unit stride in one dimension."""
    import numpy as np
    if not isinstance(X, np.ndarray) or X.ndim != 2:
        raise DimensionMismatch("%s must be a 2-D numpy array" % name)
    if out and not X.flags.writeable:
        raise ValueError("%s must be writable" % name)
    r, c = X.shape
    it = X.itemsize
    s0, s1 = X.strides
    if (s0 == it or r <= 1) and s1 % it == 0 and (c <= 1 or s1 // it >= max(1, r)):
        return X, (s1 // it if c > 1 else max(1, r)), 0
    if (s1 == it or c <= 1) and s0 % it == 0 and (r <= 1 or s0 // it >= max(1, c)):
        return X, (s0 // it if r > 1 else max(1, c)), 1
    raise ValueError("%s must have a unit stride in one dimension" % name)


def gemm_host(C, A, B, alpha=1.0, beta=0.0, *, mode="native", slices=0, return_bound=False):
    """C = alpha * A @ B + beta * C on HOST numpy arrays, in place: the blocking host-buffer call
    (gb_gemm_f64_host / gb_gemm_f32_host uploads the operands, runs the same device product and
    downloads C before returning).  Column-major and row-major arrays (and strided views with a
    unit stride in one dimension) are read without copies; results equal gemm_ on device copies
    bit for bit."""
    import numpy as np
    dt = C.dtype
    if A.dtype != dt or B.dtype != dt or dt not in (np.float64, np.float32):
        raise TypeError("gemm_host computes in float64 or float32 with one dtype, got %s, %s, %s"
                        % (A.dtype, B.dtype, dt))
    M, K = A.shape
    K2, N = B.shape
    if K2 != K or C.shape != (M, N):
        raise DimensionMismatch("A is %dx%d, B is %dx%d, C is %dx%d" % (M, K, K2, N, *C.shape))
    Cs, ldc, tc = _host_storage(C, "C", out=True)
    As, lda, ta = _host_storage(A, "A")
    Bs, ldb, tb = _host_storage(B, "B")
    L = _lib.lib()
    md = _MODES[mode] if isinstance(mode, str) else int(mode)
    bound = ctypes.c_double(0.0)
    vp = lambda X: ctypes.c_void_p(X.ctypes.data)   # noqa: E731
    if tc == 0:
        args = (ta, tb, M, N, K, alpha, vp(As), lda, vp(Bs), ldb, beta, vp(Cs), ldc)
    else:   # row-major C: C^T = B^T A^T
        args = (1 - tb, 1 - ta, N, M, K, alpha, vp(Bs), ldb, vp(As), lda, beta, vp(Cs), ldc)
    if dt == np.float64:
        rc = L.gb_gemm_f64_host(*args, md, int(slices), ctypes.byref(bound) if return_bound else None, None)
        check(rc, "gb_gemm_f64_host")
    else:
        if md != _lib.MODE_NATIVE:
            raise ValueError("Ozaki modes emulate float64; float32 runs natively")
        check(L.gb_gemm_f32_host(*args, None), "gb_gemm_f32_host")
    return (C, bound.value) if return_bound else C


def jmul_host(D, A, X):
    """jmul!(D, A, X) on host numpy arrays (blocking): D = A * X in jBLAS's per-element order."""
    return gemm_host(D, A, X, 1.0, 0.0, mode="native")


def jmul_(D, A, X, a_prefetch=7, x_prefetch=7, a_loc=3, x_loc=3, d_loc=3):
    """jmul!(D, A, X[, Val(Aprefetch_freq), Val(Xprefetch_freq), Val(A_loc), Val(X_loc), Val(D_loc)]):
    D = A * X with jBLAS's per-element FMA order (src/gemm.jl:244-246).

    The trailing arguments are jmul!'s software-prefetch distances and cache localities, CPU
    cache hints; they are checked (non-negative integers, localities 0..3) and have no GPU
    counterpart (the operands stream through shared memory)."""
    for name, v in (("a_prefetch", a_prefetch), ("x_prefetch", x_prefetch)):
        if not isinstance(v, int) or v < 0:
            raise ValueError("%s must be a non-negative integer, got %r" % (name, v))
    for name, v in (("a_loc", a_loc), ("x_loc", x_loc), ("d_loc", d_loc)):
        if not isinstance(v, int) or not 0 <= v <= 3:
            raise ValueError("%s must be a cache locality 0..3, got %r" % (name, v))
    return gemm_(D, A, X, 1.0, 0.0, mode="native")


def fastmul_(D, A, X):
    """fastmul!(D, A, X) (src/kernels.jl:202-208): the whole small product as one tile, per element
    d = a_1 x_1 then d = fma(a_n, x_n, d) — jmul!'s chain, so the same call.  Many such products
    of one shape go through gemm_strided_batched_ in one launch."""
    return gemm_(D, A, X, 1.0, 0.0, mode="native")


def kernel_raw(pD, pA, pX, Mk, Pk, stride_AD, stride_X, N, *, dtype, init=False, stream=None):
    """kernel!(pD, pA, pX, Kernel{Mk,Pk,stride_AD,stride_X,N}) on device pointers (ints)
    (src/kernels.jl:212-239): D (Mk x Pk) += A (Mk x N) * X (N x Pk), A and D with leading
    dimension stride_AD, X with stride_X, per element d = fma(a_n, x_n, d) for n = 1..N from D's
    value.  init=True is initkernel! (src/kernels.jl:240-273): D = A * X."""
    name = {torch.float64: "gb_kernel_f64", torch.float32: "gb_kernel_f32"}.get(dtype)
    if name is None:
        raise TypeError("kernel! computes in float64 or float32, got %s" % dtype)
    rc = getattr(_lib.lib(), name)(ctypes.c_void_p(pD), ctypes.c_void_p(pA), ctypes.c_void_p(pX), Mk, Pk,
                                   stride_AD, stride_X, N, int(bool(init)), ctypes.c_void_p(stream))
    check(rc, name)


def kernel_(D, A, X, init=False):
    """kernel!(D, A, X) on tensors: D (Mk x Pk) += A (Mk x N) * X (N x Pk) in jBLAS's chain
    (init=True: D = A * X, initkernel!).  D and A are column-major with the same leading
    dimension (the kernel's stride_AD), X column-major.  Returns D."""
    dt = _dtype_of(D, A, X)
    Mk, N = A.shape
    N2, Pk = X.shape
    if N2 != N or tuple(D.shape) != (Mk, Pk):
        raise DimensionMismatch("D is %dx%d, A is %dx%d, X is %dx%d" % (*D.shape, Mk, N, N2, Pk))
    Ds, ldd, td = _storage(D, "D", allow_copy=False)
    As, lda, ta = _storage(A, "A", allow_copy=False)
    Xs, ldx, tx = _storage(X, "X", allow_copy=False)
    if td or ta or tx:
        raise ValueError("kernel!: D, A and X must be column-major")
    if N > 1 and Pk > 1 and lda != ldd:
        raise ValueError("kernel!: A and D share one leading dimension (stride_AD), got %d and %d" % (lda, ldd))
    sad = ldd if Pk > 1 else (lda if N > 1 else max(1, Mk))   # the one that is used
    kernel_raw(Ds.data_ptr(), As.data_ptr(), Xs.data_ptr(), Mk, Pk, sad, ldx, N, dtype=dt, init=init,
               stream=torch.cuda.current_stream(D.device).cuda_stream)
    return D


def initkernel_(D, A, X):
    """initkernel!(D, A, X): D = A * X with d = a_1 x_1 first (src/kernels.jl:240-273)."""
    return kernel_(D, A, X, init=True)


def gemm_strided_batched_(C, A, B, alpha=1.0, beta=0.0):
    """C[i] = alpha * A[i] @ B[i] + beta * C[i] for every i, in place (jmul!'s FMA chain).

    A (count, M, K), B (count, K, N), C (count, M, N): CUDA tensors of one dtype whose
    matrices are column-major (stride 1 along rows, e.g. ``X.transpose(1, 2)`` of a
    contiguous tensor); A or B may be broadcast along the batch (stride 0).  Returns C."""
    dt = _dtype_of(C, A, B)
    cnt, M, K = A.shape
    cnt2, K2, N = B.shape
    if K2 != K or cnt2 != cnt or tuple(C.shape) != (cnt, M, N):
        raise DimensionMismatch("A %s, B %s, C %s" % (tuple(A.shape), tuple(B.shape), tuple(C.shape)))

    def batch_cm(X, rows, cols, name):
        sb, sr, sc = X.stride()
        if rows > 1 and sr != 1:
            raise ValueError("%s: matrices must be column-major (stride 1 along rows)" % name)
        return sb, (sc if cols > 1 else max(1, rows))

    sa, lda = batch_cm(A, M, K, "A")
    sb, ldb = batch_cm(B, K, N, "B")
    sc, ldc = batch_cm(C, M, N, "C")
    name = "gb_gemm_strided_batched_f64" if dt == torch.float64 else "gb_gemm_strided_batched_f32"
    st = torch.cuda.current_stream(C.device).cuda_stream
    rc = getattr(_lib.lib(), name)(M, N, K, float(alpha), ctypes.c_void_p(A.data_ptr()), max(1, lda), sa,
                                  ctypes.c_void_p(B.data_ptr()), max(1, ldb), sb, float(beta),
                                  ctypes.c_void_p(C.data_ptr()), max(1, ldc), sc, cnt, ctypes.c_void_p(st))
    check(rc, name)
    return C


_SEMIRING_FN = {torch.float64: "gb_gemm_semiring_f64", torch.float32: "gb_gemm_semiring_f32",
                torch.int32: "gb_gemm_semiring_i32"}


def gemm_semiring_(C, A, B, semiring="min_plus", accumulate=False):
    """C = [C (+)] (+)_k A[:, k] (x) B[k, :] over a semiring, in place; returns C.

    semiring: "min_plus" (shortest paths), "max_plus", "max_min" (widest paths), "min_max"
    or "max_times"; (+) is the first operation, (x) the second.  float64, float32 or int32
    CUDA tensors of one dtype.  For floating point (+) ignores NaN operands and a zero result
    is +0.0; int32 + and * wrap modulo 2^32.  accumulate=False overwrites C (an empty
    contraction gives the identity of (+)); accumulate=True folds C in with (+).  jBLAS names
    min-plus algebra as the use of its Vec fallback (src/jBLAS.jl:10).
    """
    dt = C.dtype
    if A.dtype != dt or B.dtype != dt:
        raise TypeError("all operands must share one dtype, got %s, %s, %s" % (A.dtype, B.dtype, dt))
    if dt not in _SEMIRING_FN:
        raise TypeError("semiring GEMM computes in float64, float32 or int32, got %s" % dt)
    if semiring not in _lib.SEMIRINGS:
        raise ValueError("unknown semiring %r (one of %s)" % (semiring, ", ".join(_lib.SEMIRINGS)))
    M, K = A.shape
    K2, N = B.shape
    if K2 != K or tuple(C.shape) != (M, N):
        raise DimensionMismatch("A is %dx%d, B is %dx%d, C is %dx%d" % (M, K, K2, N, *C.shape))
    Cs, ldc, tc = _storage(C, "C", allow_copy=False)
    As, lda, ta = _storage(A, "A", allow_copy=True)
    Bs, ldb, tb = _storage(B, "B", allow_copy=True)
    fn = getattr(_lib.lib(), _SEMIRING_FN[dt])
    sr = _lib.SEMIRINGS[semiring]
    st = _stream_ptr(C)
    if tc == 0:
        rc = fn(sr, ta, tb, M, N, K, ctypes.c_void_p(As.data_ptr()), lda, ctypes.c_void_p(Bs.data_ptr()), ldb,
                int(bool(accumulate)), ctypes.c_void_p(Cs.data_ptr()), ldc, st)
    else:
        # C stored row-major: C^T = B^T (x) A^T ((x) is commutative in every semiring offered)
        rc = fn(sr, 1 - tb, 1 - ta, N, M, K, ctypes.c_void_p(Bs.data_ptr()), ldb, ctypes.c_void_p(As.data_ptr()),
                lda, int(bool(accumulate)), ctypes.c_void_p(Cs.data_ptr()), ldc, st)
    check(rc, _SEMIRING_FN[dt])
    return C


def gemm_semiring(A, B, semiring="min_plus"):
    """Allocating form of gemm_semiring_: a new column-major M x N result."""
    C = torch.empty((B.shape[1], A.shape[0]), dtype=A.dtype, device=A.device).t()
    return gemm_semiring_(C, A, B, semiring)


def gemm(A, B, *, mode="native", slices=0):
    """Allocating form: returns A @ B as a new column-major tensor."""
    dt = _dtype_of(A, B)
    C = torch.empty((B.shape[1], A.shape[0]), dtype=dt, device=A.device).t()
    return gemm_(C, A, B, 1.0, 0.0, mode=mode, slices=slices)


def ozaki_plan(M, N, K, slices):
    """The slice/bit/grouping plan the Ozaki kernel uses for this shape (no GPU work)."""
    p = _lib.OzakiPlan()
    check(_lib.lib().gb_plan_ozaki(M, N, K, slices, ctypes.byref(p)), "gb_plan_ozaki")
    return {"slices": p.slices, "bits": p.bits, "k_chunk": p.k_chunk, "products": p.products,
            "groups": p.groups, "flops_tensor": p.flops_tensor}


def ozaki_crt_plan(M, N, K, moduli):
    """The CRT plan for `moduli` moduli: integer bits t ("bits"), K chunk, tensor flops."""
    p = _lib.OzakiPlan()
    check(_lib.lib().gb_plan_ozaki_crt(M, N, K, moduli, ctypes.byref(p)), "gb_plan_ozaki_crt")
    return {"moduli": p.slices, "bits": p.bits, "k_chunk": p.k_chunk, "products": p.products,
            "groups": p.groups, "flops_tensor": p.flops_tensor}


def crt_blocks(M, N, panels, sms, host_copies=False):
    """Row and column boundaries of the blocks of C a CRT call on an M x N output cuts, for the
    tuning's `panels`, a device of `sms` SMs and (host_copies) a host-buffer call with a pinned
    C (no GPU work): {"rows": [...], "cols": [...]}."""
    rows, cols = (ctypes.c_int64 * 3)(), (ctypes.c_int64 * 5)()
    nr, nc = ctypes.c_int(0), ctypes.c_int(0)
    check(_lib.lib().gb_crt_blocks(M, N, panels, sms, int(bool(host_copies)), rows, ctypes.byref(nr), cols,
                                   ctypes.byref(nc)), "gb_crt_blocks")
    return {"rows": list(rows[:nr.value + 1]), "cols": list(cols[:nc.value + 1])}


def last_ozaki_plan():
    """Plan of this thread's most recent Ozaki call (the slice count an automatic call chose)."""
    p = _lib.OzakiPlan()
    check(_lib.lib().gb_last_ozaki_plan(ctypes.byref(p)), "gb_last_ozaki_plan")
    return {"slices": p.slices, "bits": p.bits, "k_chunk": p.k_chunk, "products": p.products,
            "groups": p.groups, "flops_tensor": p.flops_tensor}


def set_ozaki_tolerance(tol):
    check(_lib.lib().gb_set_ozaki_tolerance(float(tol)), "gb_set_ozaki_tolerance")


def set_ozaki_min_chunks(n):
    """K chunking for explicit-slice Ozaki calls (wider digits for n > 1); 0/1 = default."""
    check(_lib.lib().gb_set_ozaki_min_chunks(int(n)), "gb_set_ozaki_min_chunks")


def measure_fma_peaks():
    """{"fp64_tflops", "fp32_tflops"}: the current GPU's FMA-pipe peaks, measured by a
    register-only loop (gb_measure_fma_peaks; synchronises the device)."""
    d64, d32 = ctypes.c_double(0.0), ctypes.c_double(0.0)
    check(_lib.lib().gb_measure_fma_peaks(ctypes.byref(d64), ctypes.byref(d32)), "gb_measure_fma_peaks")
    return {"fp64_tflops": d64.value, "fp32_tflops": d32.value}


def set_tc_engine(engine):
    """Tensor-core engine: 0 automatic, 1 single-CTA 128x256 tiles, 2 CTA pairs (256x256)."""
    check(_lib.lib().gb_set_tc_engine(int(engine)), "gb_set_tc_engine")


def set_wait_limit_ns(ns):
    check(_lib.lib().gb_set_wait_limit_ns(int(ns)), "gb_set_wait_limit_ns")


def check_device_status(stream=None):
    """Raises GBError if a kernel recorded a pipeline timeout since the last check."""
    s = ctypes.c_void_p(stream if stream is not None else torch.cuda.current_stream().cuda_stream)
    check(_lib.lib().gb_check_status(s), "gb_check_status")


def launch_counts():
    """{kernel kind name: launches since load} from the library's always-on counters."""
    L = _lib.lib()
    arr = (ctypes.c_longlong * _lib.KERNEL_KINDS)()
    check(L.gb_launch_counts(arr, _lib.KERNEL_KINDS), "gb_launch_counts")
    return {L.gb_kernel_kind_name(i).decode(): arr[i] for i in range(_lib.KERNEL_KINDS) if arr[i]}


class profile:
    """Context manager: CUDA-event times of every library kernel launched inside it.

    with gbblas.profile() as p: ...
    p.ms[name], p.launches[name]   summed device milliseconds and launch counts per kind
    """

    def __enter__(self):
        check(_lib.lib().gb_profile_start(), "gb_profile_start")
        self.ms, self.launches = {}, {}
        return self

    def __exit__(self, *exc):
        L = _lib.lib()
        n = _lib.KERNEL_KINDS
        ms = (ctypes.c_double * n)()
        ln = (ctypes.c_longlong * n)()
        check(L.gb_profile_stop(ms, ln, n), "gb_profile_stop")
        for i in range(n):
            if ln[i]:
                name = L.gb_kernel_kind_name(i).decode()
                self.ms[name] = ms[i]
                self.launches[name] = ln[i]
        return False


def gemm_adjoint_(dA, dB, A, B, dC):
    """dA = dC @ B^T and dB = A^T @ dC in one tensor-core launch (float32, 3xBF16 split).

    The pullback of C = A @ B (the rrule of jBLAS's jmul!/gemm!).  Inputs may be any
    2-D float32 CUDA tensors (copied to column-major if needed); dA and dB must be
    column-major and are overwritten."""
    for t in (dA, dB, A, B, dC):
        if t.dtype != torch.float32:
            raise TypeError("the adjoint kernel computes in float32")
    M, K = A.shape
    K2, N = B.shape
    if K2 != K or tuple(dC.shape) != (M, N) or tuple(dA.shape) != (M, K) or tuple(dB.shape) != (K, N):
        raise DimensionMismatch("A %s, B %s, dC %s, dA %s, dB %s" % (tuple(A.shape), tuple(B.shape),
                                tuple(dC.shape), tuple(dA.shape), tuple(dB.shape)))

    def colmajor(X, name, out=False):
        S, ld, tr = _storage(X, name, allow_copy=not out)
        if tr:
            if out:
                raise ValueError("%s must be column-major (stride (1, ld))" % name)
            S = X.t().contiguous().t()
            ld = max(1, X.shape[0])
        return S, ld

    As, lda = colmajor(A, "A")
    Bs, ldb = colmajor(B, "B")
    Cs, ldc = colmajor(dC, "dC")
    dAs, ldda = colmajor(dA, "dA", out=True)
    dBs, lddb = colmajor(dB, "dB", out=True)
    st = ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)
    rc = _lib.lib().gb_gemm_adjoint_f32(M, N, K, ctypes.c_void_p(As.data_ptr()), lda,
                                        ctypes.c_void_p(Bs.data_ptr()), ldb, ctypes.c_void_p(Cs.data_ptr()),
                                        ldc, ctypes.c_void_p(dAs.data_ptr()), ldda,
                                        ctypes.c_void_p(dBs.data_ptr()), lddb, st)
    check(rc, "gb_gemm_adjoint_f32")
    return dA, dB


def _empty_colmajor(rows, cols, like):
    return torch.empty((cols, rows), dtype=like.dtype, device=like.device).t()


class GemmFunction(torch.autograd.Function):
    """C = A @ B with the gbblas kernels forward and backward.

    The PyTorch counterpart of registering an rrule for gemm!: forward is the native
    jmul! chain (float32) or the Ozaki path (float64); backward is the fused adjoint
    kernel (float32) or two Ozaki products (float64)."""

    @staticmethod
    def forward(ctx, A, B):
        ctx.save_for_backward(A, B)
        C = _empty_colmajor(A.shape[0], B.shape[1], A)
        return gemm_(C, A, B, mode="native" if A.dtype == torch.float32 else "ozaki")

    @staticmethod
    def backward(ctx, dC):
        A, B = ctx.saved_tensors
        dA = _empty_colmajor(A.shape[0], A.shape[1], A)
        dB = _empty_colmajor(B.shape[0], B.shape[1], B)
        if A.dtype == torch.float32:
            gemm_adjoint_(dA, dB, A, B, dC.to(torch.float32))
        else:
            gemm_(dA, dC, B.t(), mode="ozaki")
            gemm_(dB, A.t(), dC, mode="ozaki")
        return dA, dB


def gemm_autograd(A, B):
    """Differentiable A @ B through GemmFunction."""
    return GemmFunction.apply(A, B)
