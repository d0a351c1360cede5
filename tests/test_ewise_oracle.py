"""Pins the oracle's restatement of the reference's unused element-wise
operations and matrix-vector products (include/matrix_la.h:272-541,
1279-1291): against the committed outputs of the reference's eWiseAdd and
VxM (tests/golden/ewise.npz), against the live reference where it was built,
and by their defining identities where the reference's code cannot run
(eWiseMult loops forever on any nonempty row, MxV does not compile)."""
import os

import numpy as np
import pytest

import oracle
from graphs import random_csr

HERE = os.path.dirname(os.path.abspath(__file__))
Z = np.load(os.path.join(HERE, "golden", "ewise.npz"))
KEYS = sorted(k[: -len("_A_rst")] for k in Z.files if k.endswith("_A_rst"))


def _csr(key, nm, n):
    rst = Z[f"{key}_{nm}_rst"]
    return oracle.Csr(len(rst) - 1, n, rst, Z[f"{key}_{nm}_col"], Z[f"{key}_{nm}_val"])


def _same(X, Y):
    return np.array_equal(X.rst, Y.rst) and np.array_equal(X.col, Y.col) and np.array_equal(
        np.asarray(X.val).view(np.uint8), np.asarray(Y.val).view(np.uint8))


@pytest.mark.parametrize("key", KEYS)
def test_golden_ewise_add_and_vxm(key):
    n = len(Z[f"{key}_y"])
    A, B, M, B2 = (_csr(key, nm, n) for nm in ("A", "B", "M", "B2"))
    assert _same(oracle.ewise_add(A, B), _csr(key, "add", n))
    assert _same(oracle.ewise_add(A, B2, M), _csr(key, "madd", n))
    assert np.array_equal(oracle.vxm(A, Z[f"{key}_x"], Z[f"{key}_y"]).view(np.uint8), Z[f"{key}_vxm"].view(np.uint8))


@pytest.mark.skipif(not oracle.ref_available(), reason="reference library not built here")
@pytest.mark.parametrize("dt", [np.int32, np.float64])
def test_live_reference_ewise_add_and_vxm(dt):
    rng = np.random.default_rng(17)
    for _ in range(4):
        A, B, M = (random_csr(70, 45, d, rng, dt) for d in (0.15, 0.25, 0.3))
        assert _same(oracle.ewise_add(A, B), oracle.ref_ewise_add(A, B))
        x = random_csr(1, 70, 1.0, rng, dt).val
        y = random_csr(1, 45, 1.0, rng, dt).val
        assert np.array_equal(oracle.vxm(A, x, y), oracle.ref_vxm(A, x, y))


def test_ewise_mult_and_mxv_identities():
    rng = np.random.default_rng(4)
    for dt in (np.int32, np.float64):
        A, B, M = (random_csr(50, 40, d, rng, dt) for d in (0.3, 0.3, 0.4))
        Ad, Bd = (np.zeros((50, 40), dt) for _ in range(2))
        Ap, Bp, Mp = (np.zeros((50, 40), bool) for _ in range(3))
        for D, P, X in ((Ad, Ap, A), (Bd, Bp, B), (None, Mp, M)):
            r = np.repeat(np.arange(50), np.diff(X.rst))
            P[r, X.col] = True
            if D is not None:
                D[r, X.col] = X.val
        both = Ap & Bp
        C = oracle.ewise_mult(A, B)
        Cd = np.zeros((50, 40), dt)
        Cp = np.zeros((50, 40), bool)
        Cd[np.repeat(np.arange(50), np.diff(C.rst)), C.col] = C.val
        Cp[np.repeat(np.arange(50), np.diff(C.rst)), C.col] = True
        assert np.array_equal(Cp, both) and np.array_equal(Cd, np.where(both, Ad * Bd, 0))
        CM = oracle.ewise_mult(A, B, M)
        assert CM.nnz == (both & Mp).sum()
        x = random_csr(1, 40, 1.0, rng, dt).val
        y0 = random_csr(1, 50, 1.0, rng, dt).val
        got = oracle.mxv(A, x, y0)
        if dt == np.int32:
            assert np.array_equal(got, y0 + Ad @ x)
        else:
            np.testing.assert_allclose(got, y0 + Ad @ x, rtol=1e-12, atol=1e-12)
        S = oracle.mult_scalar(A, 2.5)
        assert np.array_equal(S.val, (A.val.astype(np.float64) * 2.5).astype(dt))
