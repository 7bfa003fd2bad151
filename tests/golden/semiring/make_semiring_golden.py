"""Known-answer fixture for the semiring GEMM: all-pairs shortest paths.

Writes apsp_48.npz: W, the weight matrix of a seeded random digraph on 48 nodes (integer
weights 1..100, edge probability 0.12; +inf where there is no edge, 0 on the diagonal),
node 0 has no incoming and node 47 no outgoing edge, and D, its shortest-path lengths by Floyd-Warshall in Python integers (+inf where a node
is unreachable).  The (min, +) closure of W by repeated squaring must reproduce D.

    python tests/golden/semiring/make_semiring_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "..", "oracle"))
import oracle  # noqa: E402

N_NODES = 48
SEED = 20260101


def weights(n=N_NODES, seed=SEED):
    g = np.random.default_rng(seed)
    edge = g.random((n, n)) < 0.12
    w = g.integers(1, 101, (n, n))
    edge[:, 0] = False      # node 0: a source nothing reaches
    edge[n - 1, :] = False  # node n-1: a sink that reaches nothing
    return [[(int(w[i, j]) if edge[i, j] and i != j else None) for j in range(n)] for i in range(n)]


def as_float(L):
    return np.array([[np.inf if v is None else float(v) for v in row] for row in L])


def main():
    W = weights()
    D = oracle.floyd_warshall(W)
    Wf = as_float(W)
    np.fill_diagonal(Wf, 0.0)
    np.savez_compressed(os.path.join(HERE, "apsp_48.npz"), W=Wf, D=as_float(D))


if __name__ == "__main__":
    main()
