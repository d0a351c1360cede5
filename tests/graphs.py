"""Seeded test inputs (numpy) shared by the CPU and GPU tests."""
from __future__ import annotations

import numpy as np

import oracle


def dense_to_csr(D: np.ndarray, vals: np.ndarray | None = None, dtype=np.int32) -> oracle.Csr:
    m, n = D.shape
    rst = np.zeros(m + 1, np.int32)
    rst[1:] = np.cumsum((D != 0).sum(1))
    r, c = np.nonzero(D)
    val = (vals[r, c] if vals is not None else np.ones(len(c))).astype(dtype)
    return oracle.Csr(m, n, rst, c.astype(np.int32), val)


def random_csr(m: int, n: int, density: float, rng, dtype=np.int32) -> oracle.Csr:
    D = rng.random((m, n)) < density
    if np.dtype(dtype).kind in "iu":
        V = rng.integers(-3, 4, size=(m, n))
        if np.dtype(dtype) == np.uint8:
            V = rng.integers(0, 4, size=(m, n))
    else:
        V = rng.standard_normal((m, n))
    return dense_to_csr(D, V, dtype)


def random_graph(n: int, density: float, rng) -> oracle.Csr:
    """Symmetric 0/1 adjacency without self-loops."""
    U = np.triu(rng.random((n, n)) < density, 1)
    return dense_to_csr(U | U.T)


def csr_from_arrays(m: int, rst, col, dtype=np.int32) -> oracle.Csr:
    return oracle.Csr(m, m, np.asarray(rst, np.int32), np.asarray(col, np.int32), np.ones(len(col), dtype))


def to_device(ctx, A: oracle.Csr):
    import graphalgo_gb300 as ga
    return ga.Csr.upload(ctx, A.m, A.n, A.rst, A.col, A.val)
