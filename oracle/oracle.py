"""CPU oracle for the jBLAS blocked-GEMM hot path — TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU baseline arm may import
this module, and only as the checker or the timed CPU reference; the GPU product path
never calls it.

Parity status: UNPINNED by the reference's own tests (jBLAS.jl's test/runtests.jl has
no assertions, seeds or stored outputs, and the package cannot run without Julia).  The
restatements here are pinned against each other instead:
  * ``gemm`` / ``jmul``      C restatement of jmul!'s FMA chain (jmul_oracle.c), checked
                             bit-exactly against ``chain_exact`` and the committed
                             fixtures of tests/golden/ (made by make_golden.py);
  * ``chain_exact``          pure-Python restatement with exact rationals: each step
                             rounds a*b + d exactly once (CPython's int/int true division
                             is correctly rounded), following src/gemm.jl:76-89,154-168;
  * ``dot2_entries``         compensated dot products (Ogita-Rump-Oishi Dot2) for
                             near-exact values at sampled entries of large products;
  * ``quad_entries``         the same entries accumulated in IEEE binary128, the second
                             near-exact reference (pinned against exact rationals and Dot2);
  * ``ozaki_*``              numpy restatement of the Ozaki splitting and recombination
                             the GPU kernel performs, operation for operation;
  * ``semiring_gemm``        numpy restatement of the semiring product ((min, +) and its
                             relatives, the use jBLAS names for its Vec fallback,
                             src/jBLAS.jl:10), checked against ``semiring_gemm_reduce``
                             (a K-axis reduction of the full product tensor, another
                             order) and, for (min, +), against Floyd-Warshall distances
                             computed with Python integers (``floyd_warshall``).
"""
import ctypes
import math
import os
import sys
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None
c_i64 = ctypes.c_int64
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="F_CONTIGUOUS")
_vp = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        L.or_gemm_f64.argtypes = [ctypes.c_int, ctypes.c_int, c_i64, c_i64, c_i64, ctypes.c_double, _vp,
                                  c_i64, _vp, c_i64, ctypes.c_double, _vp, c_i64, ctypes.c_int]
        L.or_gemm_f32.argtypes = [ctypes.c_int, ctypes.c_int, c_i64, c_i64, c_i64, ctypes.c_float, _vp,
                                  c_i64, _vp, c_i64, ctypes.c_float, _vp, c_i64, ctypes.c_int]
        for nm in ("or_jmul_tiled_rc_f64", "or_jmul_tiled_rc_f32"):
            getattr(L, nm).argtypes = [ctypes.c_int, ctypes.c_int, c_i64, c_i64, c_i64, _vp, c_i64, _vp, c_i64,
                                       _vp, c_i64, ctypes.c_int]
            getattr(L, nm).restype = ctypes.c_int
        L.or_pick_kernel_size.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _vp, _vp]
        L.or_pick_kernel_size.restype = ctypes.c_int
        L.or_time_jmul_tiled_f64.argtypes = [ctypes.c_int, ctypes.c_int, c_i64, c_i64, c_i64, _vp, _vp, _vp,
                                             ctypes.c_int, ctypes.c_int]
        L.or_time_jmul_tiled_f64.restype = ctypes.c_double
        L.or_dot2_entries.argtypes = [ctypes.c_int, ctypes.c_int, c_i64, _vp, c_i64, _vp, c_i64, c_i64,
                                      _vp, _vp, _vp, _vp, _vp, ctypes.c_int]
        L.or_quad_entries.argtypes = [ctypes.c_int, ctypes.c_int, c_i64, _vp, c_i64, _vp, c_i64, c_i64, _vp,
                                      _vp, _vp, _vp, ctypes.c_int]
        L.or_fma_array.argtypes = [c_i64, _vp, _vp, _vp, _vp]
        for nm in ("or_kernel_f64", "or_kernel_f32"):
            getattr(L, nm).argtypes = [_vp, _vp, _vp, c_i64, c_i64, c_i64, c_i64, c_i64, ctypes.c_int]
        L.or_chain_entries_f64.argtypes = [ctypes.c_int, ctypes.c_int, c_i64, ctypes.c_double, _vp, c_i64,
                                           _vp, c_i64, ctypes.c_double, _vp, c_i64, c_i64, _vp, _vp, _vp,
                                           ctypes.c_int]
        L.or_chain_entries_f32.argtypes = [ctypes.c_int, ctypes.c_int, c_i64, ctypes.c_float, _vp, c_i64,
                                           _vp, c_i64, ctypes.c_float, _vp, c_i64, c_i64, _vp, _vp, _vp,
                                           ctypes.c_int]
        L.or_num_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_vp)


def _colmajor(X, dtype):
    """(array, ld) for a 2-D array stored column-major (copying if needed)."""
    X = np.asarray(X)
    if X.dtype != dtype:
        X = X.astype(dtype)
    if not X.flags.f_contiguous:
        X = np.asfortranarray(X)
    return X, max(1, X.shape[0])


def num_threads():
    return lib().or_num_threads()


def gemm(A, B, C=None, alpha=1.0, beta=0.0, trans_a=False, trans_b=False, dtype=np.float64,
         nthreads=None):
    """alpha*op(A)*op(B) + beta*C with jmul!'s element order; returns a new F-ordered array.

    A, B are the STORED matrices (op applied by the flags), as in BLAS."""
    A, lda = _colmajor(A, dtype)
    B, ldb = _colmajor(B, dtype)
    M = A.shape[1] if trans_a else A.shape[0]
    K = A.shape[0] if trans_a else A.shape[1]
    N = B.shape[0] if trans_b else B.shape[1]
    out = np.zeros((M, N), dtype=dtype, order="F") if C is None else np.array(C, dtype=dtype, order="F")
    nt = nthreads or num_threads()
    fn = lib().or_gemm_f64 if dtype == np.float64 else lib().or_gemm_f32
    fn(int(trans_a), int(trans_b), M, N, K, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(out),
       max(1, M), nt)
    return out


def jmul(A, X, dtype=np.float64):
    """jmul!(D, A, X) restated: D = A * X (src/gemm.jl:244)."""
    return gemm(A, X, dtype=dtype)


def kernel_chain(D, A, X, Mk, Pk, stride_AD, stride_X, N, init=False, dtype=np.float64):
    """jBLAS's kernel! / initkernel! on flat column-major buffers (src/kernels.jl:212-273):
    D (Mk x Pk, leading dimension stride_AD) += A (Mk x N, stride_AD) * X (N x Pk, stride_X),
    per element d = fma(a_n, x_n, d) for n = 1..N from D's value; init: D = A * X with
    d = a_1 x_1 first.  Returns the new D buffer (a copy)."""
    D = np.array(D, dtype=dtype).ravel(order="K")
    A = np.ascontiguousarray(np.asarray(A, dtype=dtype).ravel(order="K"))
    X = np.ascontiguousarray(np.asarray(X, dtype=dtype).ravel(order="K"))
    fn = lib().or_kernel_f64 if np.dtype(dtype) == np.float64 else lib().or_kernel_f32
    fn(_ptr(D), _ptr(A), _ptr(X), Mk, Pk, stride_AD, stride_X, N, int(bool(init)))
    return D


def pick_kernel_size(t_size, register_size, register_count):
    """jBLAS's micro-tile choice (src/kernel_structure.jl:76-99) restated: (elements per
    register, rows, cols) for elements of t_size bytes in register_count registers of
    register_size bytes.  Rows grow one register of A at a time; the tile gets the columns
    that the remaining registers hold beside one X broadcast register, (count - a - 1) // a;
    the search stops at the first shape whose elements per loaded register (rows * cols /
    (cols + a)) falls below the previous one's."""
    epr = register_size // t_size
    lines = -(-(epr * register_count) // epr)
    best, rows, cols = -math.inf, 0, 0
    for a in range(1, lines + 1):
        r, c = a * epr, (register_count - a - 1) // a
        ratio = (r * c) / (c + a)
        if ratio < best:
            break
        best, rows, cols = ratio, r, c
    return epr, rows, cols


def host_register_file():
    """(register bytes, register count) of this host's SIMD file, as the reference's build
    script reads them (deps/build.jl:3-4: simdbytes(), 32 registers with AVX-512F else 16):
    x86-64 AVX-512F 64 x 32, AVX2 32 x 16, SSE 16 x 16; AArch64 NEON (and 128-bit SVE) 16 x 32."""
    import platform
    if platform.machine() in ("x86_64", "AMD64"):
        flags = set()
        try:
            with open("/proc/cpuinfo") as f:
                for line in f:
                    if line.startswith("flags"):
                        flags = set(line.split())
                        break
        except OSError:
            pass
        if "avx512f" in flags:
            return 64, 32
        if "avx2" in flags:
            return 32, 16
        return 16, 16
    return 16, 32


def host_tile(dtype=np.float64):
    """(rows, cols) of the register tile pick_kernel_size gives on this host."""
    _, r, c = pick_kernel_size(np.dtype(dtype).itemsize, *host_register_file())
    return r, c


def jmul_tiled(A, B, nthreads=1, dtype=np.float64, out=None, tile=None):
    """The timed CPU baseline: jmul!'s register-tiled loop nest (same results as jmul) with the
    register tile pick_kernel_size gives for this host (or `tile` = (rows, cols))."""
    A, lda = _colmajor(A, dtype)
    B, ldb = _colmajor(B, dtype)
    M, K = A.shape
    N = B.shape[1]
    if out is None:
        out = np.empty((M, N), dtype=dtype, order="F")
    tr, tc = tile or host_tile(dtype)
    fn = lib().or_jmul_tiled_rc_f64 if np.dtype(dtype) == np.float64 else lib().or_jmul_tiled_rc_f32
    if fn(tr, tc, M, N, K, _ptr(A), lda, _ptr(B), ldb, _ptr(out), max(1, M), int(nthreads)) != 0:
        raise ValueError("no %dx%d register tile for %s" % (tr, tc, np.dtype(dtype).name))
    return out


def time_jmul_tiled(A, B, tile=None, reps=2000, batches=50):
    """Minimum time (ns) of one single-threaded float64 jmul_tiled call on A (M x K) and B (K x N),
    over `batches` batches of `reps` calls (BenchmarkTools' minimum, test/runtests.jl:111-116)."""
    A, _ = _colmajor(A, np.float64)
    B, _ = _colmajor(B, np.float64)
    M, K = A.shape
    N = B.shape[1]
    C = np.empty((M, N), order="F")
    tr, tc = tile or host_tile(np.float64)
    ns = lib().or_time_jmul_tiled_f64(tr, tc, M, N, K, _ptr(A), _ptr(B), _ptr(C), int(reps), int(batches))
    if ns < 0:
        raise ValueError("no %dx%d float64 register tile" % (tr, tc))
    return ns


def chain_entries(A, B, rows, cols, C=None, alpha=1.0, beta=0.0, trans_a=False, trans_b=False,
                  dtype=np.float64, nthreads=None):
    """jmul!'s exact per-element result (with alpha/beta) at sampled (rows[s], cols[s])."""
    A, lda = _colmajor(A, dtype)
    B, ldb = _colmajor(B, dtype)
    K = A.shape[0] if trans_a else A.shape[1]
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    if C is None:
        C0, ldc = np.zeros((1, 1), dtype=dtype, order="F"), 1
    else:
        C0, ldc = _colmajor(C, dtype)
    out = np.empty(rows.size, dtype=dtype)
    fn = lib().or_chain_entries_f64 if dtype == np.float64 else lib().or_chain_entries_f32
    fn(int(trans_a), int(trans_b), K, alpha, _ptr(A), lda, _ptr(B), ldb, beta, _ptr(C0), ldc, rows.size,
       _ptr(rows), _ptr(cols), _ptr(out), nthreads or num_threads())
    return out


def dot2_entries(A, B, rows, cols, trans_a=False, trans_b=False, nthreads=None):
    """Near-exact (hi, lo, sum|a||b|) of (op(A) op(B))[rows[s], cols[s]] via Dot2."""
    A, lda = _colmajor(A, np.float64)
    B, ldb = _colmajor(B, np.float64)
    K = A.shape[0] if trans_a else A.shape[1]
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    n = rows.size
    hi = np.empty(n)
    lo = np.empty(n)
    ab = np.empty(n)
    lib().or_dot2_entries(int(trans_a), int(trans_b), K, _ptr(A), lda, _ptr(B), ldb, n, _ptr(rows),
                          _ptr(cols), _ptr(hi), _ptr(lo), _ptr(ab), nthreads or num_threads())
    return hi, lo, ab


def quad_entries(A, B, rows, cols, trans_a=False, trans_b=False, nthreads=None):
    """(hi, lo) of (op(A) op(B))[rows[s], cols[s]] accumulated in IEEE binary128 (__float128 /
    AArch64 long double): |hi + lo - exact| <= K 2^-113 sum |a||b| (+ the final rounding to a
    double-double).  The second near-exact reference beside ``dot2_entries``."""
    A, lda = _colmajor(A, np.float64)
    B, ldb = _colmajor(B, np.float64)
    K = A.shape[0] if trans_a else A.shape[1]
    rows = np.ascontiguousarray(rows, dtype=np.int64)
    cols = np.ascontiguousarray(cols, dtype=np.int64)
    n = rows.size
    hi = np.empty(n)
    lo = np.empty(n)
    lib().or_quad_entries(int(trans_a), int(trans_b), K, _ptr(A), lda, _ptr(B), ldb, n, _ptr(rows), _ptr(cols),
                          _ptr(hi), _ptr(lo), nthreads or num_threads())
    return hi, lo


def fma(a, b, c):
    """Elementwise fused multiply-add with one rounding (float64 arrays)."""
    a, b, c = (np.ascontiguousarray(np.broadcast_to(x, np.broadcast(a, b, c).shape), dtype=np.float64)
               for x in (a, b, c))
    out = np.empty_like(a)
    lib().or_fma_array(a.size, _ptr(a), _ptr(b), _ptr(c), _ptr(out))
    return out


# ------------------------------------------------------------------ exact restatement

def _round_to_float(q: Fraction, bits: int) -> float:
    """Round a rational to the nearest binary float with `bits` significand bits
    (ties to even), IEEE range of float64 (bits=53) or float32 (bits=24)."""
    if q == 0:
        return 0.0
    if bits == 53:
        return q.numerator / q.denominator  # correctly rounded in CPython
    emin, emax = -126, 127
    sign = -1.0 if q < 0 else 1.0
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    e = max(e, emin)
    scale = Fraction(2) ** (bits - 1 - e)
    m = a * scale
    n = m.numerator // m.denominator
    rem = m - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n % 2 == 1):
        n += 1
    v = Fraction(n) / scale
    if v >= Fraction(2) ** (emax + 1):
        return sign * math.inf
    return sign * float(v)


def chain_exact(A, X, bits=53, D0=None):
    """D = A*X with each step d = round(a*x + d) evaluated exactly (pure Python, slow).

    d = a1*x1 (rounded), then d = fma(ak, xk, d) for k = 2..K (src/gemm.jl:76-89,154-168).
    With D0 (kernel!, src/kernels.jl:212-238): d starts at D0[i, j] and every k is an fma.
    Signed zeros follow IEEE: round(-0) keeps the sign of an exact zero sum as fma does."""
    A = np.asarray(A, dtype=np.float64)
    X = np.asarray(X, dtype=np.float64)
    M, K = A.shape
    P = X.shape[1]
    D = np.zeros((M, P), dtype=np.float64, order="F")
    for j in range(P):
        for i in range(M):
            if D0 is not None:
                d, k_first = float(D0[i, j]), 0
            elif K == 0:
                D[i, j] = 0.0
                continue
            else:
                d = _round_to_float(Fraction(A[i, 0]) * Fraction(X[0, j]), bits)
                if d == 0.0:
                    d = math.copysign(0.0, A[i, 0]) * math.copysign(1.0, X[0, j])
                k_first = 1
            for k in range(k_first, K):
                exact = Fraction(A[i, k]) * Fraction(X[k, j]) + Fraction(d)
                r = _round_to_float(exact, bits)
                if r == 0.0:
                    prod_sign = math.copysign(1.0, A[i, k]) * math.copysign(1.0, X[k, j])
                    if exact == 0 and prod_sign < 0 and math.copysign(1.0, d) < 0:
                        r = -0.0  # (-0) + (-0) = -0; any other exact zero sum is +0
                    elif exact == 0:
                        r = 0.0
                    else:
                        r = math.copysign(0.0, float(exact))
                d = r
            D[i, j] = d
    return D


# ------------------------------------------------------------------ Ozaki restatement

def ozaki_bits_for(kc):
    lg = 0
    while (1 << lg) < kc:
        lg += 1
    return min(9, (26 - lg) // 2)


def ozaki_plan(K, slices, min_chunks=1):
    """Same plan as the GPU planner: bits, K chunks of 64-wide panels, groups of pairs.

    min_chunks > 1 cuts K into at least that many exact chunks (wider digits), as the
    automatic slice choice may do."""
    kb_total = max(1, (K + 63) // 64)
    nchunks = max(1, (K + 65535) // 65536, min_chunks)
    nchunks = min(nchunks, kb_total)
    kb_chunk = (kb_total + nchunks - 1) // nchunks
    nchunks = (kb_total + kb_chunk - 1) // kb_chunk
    kc = kb_chunk * 64
    if kc > K:
        kc = max(1, K)
    bits = ozaki_bits_for(kc)
    share = max(1, min(8, int(math.floor(16777216.0 / (kc * 2.0 ** (2 * bits - 2))))))
    groups = []
    for level in range(slices + 1, 1, -1):   # smallest contributions first
        cur = None
        for p in range(1, slices + 1):
            q = level - p
            if q < 1 or q > slices:
                continue
            if cur is None or len(cur[1]) == share:
                cur = (level, [])
                groups.append(cur)
            cur[1].append((p - 1, q - 1))
    return {"bits": bits, "kb_chunk": kb_chunk, "kb_total": kb_total, "nchunks": nchunks,
            "k_chunk": kc, "groups": groups,
            "products": sum(len(g[1]) for g in groups)}


def ozaki_split(X, slices, bits):
    """Digits (slices, R, K) and exponents (R,) of the rows of X (R x K float64).

    Row exponent e: max|x| < 2^e.  Y = round-half-away(x * 2^(s*b - 1 - e)) is an integer;
    the digits are its balanced base-2^b expansion from the least significant end
    (d_s..d_2 in [-2^(b-1), 2^(b-1)), d_1 the remaining top part), so that
    x * 2^-e = sum_p d_p 2^(1 - p*b) + delta with |delta| <= 2^-(s*b)."""
    X = np.asarray(X, dtype=np.float64)
    R, K = X.shape
    nonfinite = ~np.isfinite(X).all(axis=1) if K else np.zeros(R, bool)
    amax = np.abs(X).max(axis=1) if K else np.zeros(R)
    _, ex = np.frexp(np.where(nonfinite, 1.0, amax))
    e = np.where(amax == 0, 0, ex).astype(np.int64)
    e_safe = np.where(nonfinite, 0, e)
    e = np.where(nonfinite, 2**31 - 1, e)
    SB = slices * bits
    H, MASK = 1 << (bits - 1), (1 << bits) - 1
    v = np.ldexp(np.where(nonfinite[:, None], 0.0, X), (SB - 1 - e_safe)[:, None].astype(np.int32))
    mag = np.abs(v)
    fl = np.floor(mag)
    ymag = fl + (mag - fl >= 0.5)
    digits = np.empty((slices, R, K))
    if SB <= 62:
        Y = (np.sign(v) * ymag).astype(np.int64)
        for p in range(slices - 1, 0, -1):
            d = ((Y + H) & MASK) - H
            Y = (Y - d) >> bits
            digits[p] = d
        digits[0] = Y
    else:
        Y = np.array([[int(a) for a in row] for row in (np.sign(v) * ymag)], dtype=object).reshape(R, K)
        for p in range(slices - 1, 0, -1):
            d = ((Y + H) & MASK) - H
            Y = (Y - d) >> bits
            digits[p] = d.astype(np.float64)
        digits[0] = Y.astype(np.float64)
    return digits, e


def chunks_for(K, k_chunk):
    """min_chunks that reproduces a plan's K chunk (as reported by the library)."""
    kb_total = max(1, (K + 63) // 64)
    kb_chunk = max(1, (k_chunk + 63) // 64)
    return max(1, (kb_total + kb_chunk - 1) // kb_chunk)


def ozaki_gemm(A, B, C=None, alpha=1.0, beta=0.0, slices=8, min_chunks=1):
    """The GPU Ozaki result restated in numpy (A: M x K, B: K x N logical operands)."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    M, K = A.shape
    N = B.shape[1]
    plan = ozaki_plan(K, slices, min_chunks)
    bits = plan["bits"]
    dA, ea = ozaki_split(A, slices, bits)
    dB, eb = ozaki_split(B.T, slices, bits)
    steps = len(plan["groups"]) * plan["nchunks"]
    T = None
    kc = plan["kb_chunk"] * 64
    for level, pairs in plan["groups"]:
        w = 2.0 ** (2 - level * bits)
        for c in range(plan["nchunks"]):
            k0, k1 = c * kc, min(K, (c + 1) * kc)
            S = np.zeros((M, N))
            for p, q in pairs:
                S += dA[p][:, k0:k1] @ dB[q][:, k0:k1].T   # exact: integers below 2^53
            T = S * w if T is None else T + S * w           # fma(S, w, T) with S*w exact
    del steps
    bad = (ea[:, None] == 2**31 - 1) | (eb[None, :] == 2**31 - 1)
    E = np.where(bad, 0, ea[:, None] + eb[None, :])
    val = np.ldexp(T, E.astype(np.int64))
    val = np.where(bad, np.nan, val)
    if beta == 0.0:
        out = alpha * val
    else:
        out = fma(np.full_like(val, alpha), val, beta * np.asarray(C, dtype=np.float64))
    return np.asfortranarray(out)


# ------------------------------------------------------------------ CRT (Ozaki scheme II)

CRT_MAX_MODULI = 20


def crt_moduli(n):
    """The first n moduli: 253, then descending integers coprime to all taken so far."""
    out, c = [], 253
    while len(out) < n:
        if all(math.gcd(c, m) == 1 for m in out):
            out.append(c)
        c -= 1
    return out


def crt_bits_for(K, n):
    """Largest t <= 62 with 4 K 2^(2t) <= prod(moduli) and K 2^(2t) <= 2^125 (0: none)."""
    Mp = math.prod(crt_moduli(n))
    K = max(1, K)
    for t in range(62, 0, -1):
        if 4 * K * 4 ** t <= Mp and K * 4 ** t <= 2 ** 125:
            return t
    return 0


def _fixed_rows(X, t):
    """Row exponents e (max|x| < 2^e; Inf/NaN rows flagged) and Y = round-half-away(x 2^(t-e))
    as int64 (|Y| <= 2^t), the integer operand of the CRT product."""
    X = np.asarray(X, dtype=np.float64)
    R, K = X.shape
    nonfinite = ~np.isfinite(X).all(axis=1) if K else np.zeros(R, bool)
    amax = np.abs(np.where(nonfinite[:, None], 0.0, X)).max(axis=1) if K else np.zeros(R)
    _, ex = np.frexp(amax)
    e = np.where(amax == 0, 0, ex).astype(np.int64)
    v = np.ldexp(np.where(nonfinite[:, None], 0.0, X), (t - e)[:, None].astype(np.int32))
    mag = np.abs(v)
    fl = np.floor(mag)
    Y = (np.sign(v) * (fl + (mag - fl >= 0.5))).astype(np.int64)
    return Y, np.where(nonfinite, 2**31 - 1, e)


def _exact_int_product(Ya, Yb):
    """Exact integer Ya @ Yb.T (|entries| <= 2^62, K <= 2^19) as an object array of Python
    ints.  The operands are cut into 17-bit limbs (the top one signed, |.| <= 2^11), so every
    partial sum of a limb product is an integer below 2^53 and the float64 matrix products
    are exact in any summation order."""
    def limbs(Y):
        out = []
        for _ in range(3):
            out.append((Y & ((1 << 17) - 1)).astype(np.float64))
            Y = Y >> 17
        out.append(Y.astype(np.float64))
        return out
    if Ya.shape[1] > (1 << 19):
        raise ValueError("K too large for the exact limb product")
    la, lb = limbs(Ya), limbs(Yb)
    total = None
    for d in range(7):
        S = None
        for l in range(4):
            m = d - l
            if 0 <= m < 4:
                P = (la[l] @ lb[m].T).astype(np.int64)
                S = P if S is None else S + P
        term = S.astype(object) * (1 << (17 * d))
        total = term if total is None else total + term
    return total


def ozaki_crt_gemm(A, B, C=None, alpha=1.0, beta=0.0, moduli=16, bits=0):
    """The GPU CRT-mode result restated: C = alpha * fl(A'B' 2^(ea+eb-2t)) + beta * C with
    A', B' the t-bit integer operands and A'B' computed exactly (no residues needed for the
    restatement: the CRT reconstruction on the GPU must give this exact product)."""
    A = np.asarray(A, dtype=np.float64)
    B = np.asarray(B, dtype=np.float64)
    M, K = A.shape
    N = B.shape[1]
    t = bits or crt_bits_for(K, moduli)
    Ya, ea = _fixed_rows(A, t)
    Yb, eb = _fixed_rows(B.T, t)
    Cint = _exact_int_product(Ya, Yb) if K else np.zeros((M, N), dtype=object)
    T = np.array([float(v) for v in Cint.ravel()], dtype=np.float64).reshape(M, N)
    bad = (ea[:, None] == 2**31 - 1) | (eb[None, :] == 2**31 - 1)
    E = np.where(bad, 0, ea[:, None] + eb[None, :] - 2 * t)
    val = np.where(bad, np.nan, np.ldexp(T, E.astype(np.int64)))
    if beta == 0.0:
        out = alpha * val
    else:
        out = fma(np.full_like(val, alpha), val, beta * np.asarray(C, dtype=np.float64))
    return np.asfortranarray(out)


# ---------------------------------------------------------------------------- semirings
SEMIRINGS = ("min_plus", "max_plus", "max_min", "min_max", "max_times")


def _semiring_ops(semiring, dtype):
    """(oplus, otimes, identity of oplus) for one semiring and element type.

    Floating point: oplus is min/max ignoring NaN operands (np.fmin / np.fmax); otimes
    is +, *, or the same NaN-ignoring min/max, rounded to nearest in `dtype`.  int32:
    + and * wrap modulo 2^32 (numpy array arithmetic), min/max are exact."""
    if semiring not in SEMIRINGS:
        raise ValueError("unknown semiring %r" % (semiring,))
    is_int = np.issubdtype(dtype, np.integer)
    mn = np.minimum if is_int else np.fmin
    mx = np.maximum if is_int else np.fmax
    if semiring in ("min_plus", "min_max"):
        oplus, ident = mn, (np.iinfo(dtype).max if is_int else np.inf)
    else:
        oplus, ident = mx, (np.iinfo(dtype).min if is_int else -np.inf)
    otimes = {"min_plus": np.add, "max_plus": np.add, "max_min": mn, "min_max": mx,
              "max_times": np.multiply}[semiring]
    return oplus, otimes, dtype.type(ident)


def _semiring_finish(acc, dtype):
    if not np.issubdtype(dtype, np.integer):
        acc[acc == 0] = 0   # a zero result is +0.0 (removes the K-order dependence of its sign)
    return acc


def semiring_gemm(A, B, semiring, C=None, accumulate=False, dtype=np.float64):
    """C = [C (+)] (+)_k A[:, k] (x) B[k, :], folding k = 1..K in order (the sequential
    K loop of jmul!'s register tile, src/gemm.jl:149-170, with the semiring's operations
    in place of fma).  Returns a new array of `dtype`; K = 0 gives the identity of (+)."""
    dtype = np.dtype(dtype)
    A = np.asarray(A, dtype=dtype)
    B = np.asarray(B, dtype=dtype)
    M, K = A.shape
    N = B.shape[1]
    oplus, otimes, ident = _semiring_ops(semiring, dtype)
    acc = np.full((M, N), ident, dtype=dtype)
    with np.errstate(all="ignore"):
        for k in range(K):
            acc = oplus(acc, otimes(A[:, k:k + 1], B[k:k + 1, :]))
        if accumulate:
            acc = oplus(np.asarray(C, dtype=dtype), acc)
    return _semiring_finish(np.asfortranarray(acc), dtype)


def semiring_gemm_reduce(A, B, semiring, dtype=np.float64):
    """The same product as one reduction over the K axis of the M x K x N tensor of (x)
    products (numpy's pairwise reduction order): a second order for pinning ``semiring_gemm``
    (small sizes only)."""
    dtype = np.dtype(dtype)
    A = np.asarray(A, dtype=dtype)
    B = np.asarray(B, dtype=dtype)
    oplus, otimes, ident = _semiring_ops(semiring, dtype)
    with np.errstate(all="ignore"):
        T = otimes(A[:, :, None], B[None, :, :])
        acc = oplus.reduce(T, axis=1, initial=ident)
    return _semiring_finish(np.asfortranarray(acc), dtype)


def floyd_warshall(W):
    """All-pairs shortest path lengths of a weighted digraph given as a list of lists of
    Python ints (None = no edge), by Floyd-Warshall in exact integers; None = unreachable."""
    n = len(W)
    D = [[(0 if i == j else W[i][j]) for j in range(n)] for i in range(n)]
    for k in range(n):
        Dk = D[k]
        for i in range(n):
            dik = D[i][k]
            if dik is None:
                continue
            Di = D[i]
            for j in range(n):
                if Dk[j] is not None and (Di[j] is None or dik + Dk[j] < Di[j]):
                    Di[j] = dik + Dk[j]
    return D
