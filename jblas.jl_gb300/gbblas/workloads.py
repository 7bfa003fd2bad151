"""Seeded synthetic inputs for the five benchmark workloads (numpy, portable).

numpy's PCG64 generator gives the same streams on x86_64 and aarch64, so a seed names
the same matrices on every machine.  Matrices are returned column-major
(Fortran-ordered), the layout jBLAS's MMatrix uses.

  plain   uniform[-1, 1) entries (the 256^3 case and the 1024..16384 sweep)
  ozaki   sign * U[1,2) * 2^(e_line + e_elem), e_line uniform integer in [-30, 30] per
          row of A / column of B, e_elem uniform integer in [-8, 8] per element
  grouped m, n, k each round(exp(U[ln 8, ln 512])) for 4096 independent problems
  adjoint A 4096x2048, B 2048x4096, W 4096x4096 float32 N(0, 1)
"""
import numpy as np

SEED = 20260101


def rng(seed=SEED, stream=0):
    return np.random.Generator(np.random.PCG64([seed, stream]))


def uniform(m, n, seed=SEED, stream=0, dtype=np.float64):
    """m x n column-major matrix of uniform[-1, 1) entries."""
    g = rng(seed, stream)
    x = g.random((n, m), dtype=np.float64)
    x *= 2.0
    x -= 1.0
    return x.astype(dtype, copy=False).T  # (m, n) view, Fortran-ordered


def ozaki_matrix(m, n, *, per="row", seed=SEED, stream=0, e_line=30, e_elem=8):
    """sign * U[1,2) * 2^(e_line_i + e_elem_ij); per = "row" (A) or "col" (B)."""
    g = rng(seed, stream)
    mant = g.random((n, m)) + 1.0
    sign = np.where(g.random((n, m)) < 0.5, -1.0, 1.0)
    ee = g.integers(-e_elem, e_elem + 1, size=(n, m))
    if per == "row":
        el = g.integers(-e_line, e_line + 1, size=m)[None, :]
    else:
        el = g.integers(-e_line, e_line + 1, size=n)[:, None]
    x = np.ldexp(sign * mant, (ee + el).astype(np.int32))
    return x.T


def grouped_sizes(count=4096, lo=8, hi=512, seed=SEED, stream=7):
    """(count, 3) int64 array of (m, n, k), each round(exp(U[ln lo, ln hi]))."""
    g = rng(seed, stream)
    v = np.rint(np.exp(g.uniform(np.log(lo), np.log(hi), size=(count, 3))))
    return v.astype(np.int64)


def normal(m, n, seed=SEED, stream=0, dtype=np.float32):
    g = rng(seed, stream)
    return g.standard_normal((n, m), dtype=np.float64).astype(dtype).T
