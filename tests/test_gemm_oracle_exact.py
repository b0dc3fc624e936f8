"""The FP64 GEMM oracle (numpy float64 matmul, used by the GEMM parity tests)
bounded by exact rational dot products on sampled entries of a C3-shaped
contraction (Bm^T Bm, Bm[p, q] = N(0,1) exp(-0.01 p)): its own relative error
must be far below the 1e-12 bar the Ozaki GEMM is held to."""

from fractions import Fraction

import numpy as np


def exact_entries(bm, pairs):
    cols = {j: [Fraction(float(x)) for x in bm[:, j]] for pair in pairs for j in pair}
    return np.array([float(sum(a * b for a, b in zip(cols[i], cols[j]))) for i, j in pairs])


def test_fp64_oracle_error_far_below_the_bar():
    rng = np.random.default_rng(0)
    P, Q = 1000, 256
    bm = rng.standard_normal((P, Q)) * np.exp(-0.01 * np.arange(P))[:, None]
    ref = bm.T @ bm
    pairs = [tuple(int(v) for v in rng.integers(0, Q, 2)) for _ in range(24)]
    exact = exact_entries(bm, pairs)
    approx = np.array([ref[i, j] for i, j in pairs])
    rel = np.linalg.norm(approx - exact) / np.linalg.norm(exact)
    assert rel < 1e-14
