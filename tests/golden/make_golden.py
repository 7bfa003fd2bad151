"""Generates the committed golden fixtures for jmul!'s arithmetic.

jBLAS.jl ships no golden vectors (test/runtests.jl runs jmul! and mul! on unseeded
random MMatrix values and discards the outputs), so the fixtures here are made from an
independent exact-rational restatement of jmul!'s per-element FMA chain
(``oracle.chain_exact``: d = a1*x1, d = fma(ak, xk, d), each step rounded once) on
seeded inputs.  Shapes are the ones the reference's benchmark script exercises
(test/runtests.jl:12-36, 103-105): M x N x P with N the contraction dimension.

Run:  python tests/golden/make_golden.py      (writes tests/golden/*.npz)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

# (name, M, N (contraction), P, dtype, distribution)
CASES = [
    ("f64_24x18x18_normal", 24, 18, 18, "f64", "normal"),
    ("f64_16x32x14_normal", 16, 32, 14, "f64", "normal"),
    ("f64_13x12x12_uniform", 13, 12, 12, "f64", "uniform"),
    ("f64_8x8x8_uniform", 8, 8, 8, "f64", "uniform"),
    ("f64_49x49x49_normal", 49, 49, 49, "f64", "normal"),
    ("f64_37x37x37_uniform", 37, 37, 37, "f64", "uniform"),
    ("f64_32x36x36_normal", 32, 36, 36, "f64", "normal"),
    ("f64_32x32x6_uniform", 32, 32, 6, "f64", "uniform"),
    ("f32_16x32x14_normal", 16, 32, 14, "f32", "normal"),
    ("f32_13x12x12_uniform", 13, 12, 12, "f32", "uniform"),
    ("f32_37x37x37_normal", 37, 37, 37, "f32", "normal"),
    ("f64_9x7x5_special", 9, 7, 5, "f64", "special"),
]


def inputs(M, N, P, dtype, dist, seed):
    g = np.random.Generator(np.random.PCG64(seed))
    np_dt = np.float64 if dtype == "f64" else np.float32
    if dist == "normal":
        A = g.standard_normal((M, N))
        X = g.standard_normal((N, P))
    elif dist == "uniform":
        A = g.uniform(-1, 1, (M, N))
        X = g.uniform(-1, 1, (N, P))
    else:
        # signed zeros, exact cancellations, tiny and huge magnitudes
        A = g.uniform(-1, 1, (M, N))
        X = g.uniform(-1, 1, (N, P))
        A[0, :] = -0.0
        A[1, :] = 0.0
        X[:, 0] = -0.0
        A[2, :] = 1.0
        X[:, 1] = np.array([1.0, -1.0] * N)[:N]
        A[3, :] = np.ldexp(1.0, -1070)
        A[4, :] = np.ldexp(1.5, 600)
        X[:, 2] = np.ldexp(1.25, 400)
        A[5, 0] = 1e-300
        X[0, 3] = -1e-300
    return np.asfortranarray(A.astype(np_dt)), np.asfortranarray(X.astype(np_dt))


def main():
    for idx, (name, M, N, P, dt, dist) in enumerate(CASES):
        A, X = inputs(M, N, P, dt, dist, seed=1000 + idx)
        bits = 53 if dt == "f64" else 24
        D = oracle.chain_exact(A.astype(np.float64), X.astype(np.float64), bits=bits)
        np_dt = np.float64 if dt == "f64" else np.float32
        np.savez_compressed(os.path.join(HERE, name + ".npz"), A=A, X=X, D=D.astype(np_dt))
        print(name, D.shape)


if __name__ == "__main__":
    main()
