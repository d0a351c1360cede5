"""Sparse element-wise operations and matrix-vector products on the GPU
against the oracle's restatement (pinned to the reference's eWiseAdd and
VxM): patterns and values bit-exact, for int32 and float64."""
import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle
from graphs import random_csr, to_device

pytestmark = pytest.mark.gpu


def check(D, E):
    rst, col, val = D.download()
    assert np.array_equal(rst, E.rst) and np.array_equal(col, E.col[: E.nnz])
    assert np.array_equal(val.view(np.uint8), np.asarray(E.val[: E.nnz], val.dtype).view(np.uint8))


def hub_csr(m, n, rng, dt, hub_row=3):
    """Random sparse matrix with one dense row (a hub)."""
    A = random_csr(m, n, 0.02, rng, dt)
    D = np.zeros((m, n), bool)
    D[np.repeat(np.arange(m), np.diff(A.rst)), A.col] = True
    D[hub_row, :] = rng.random(n) < 0.7
    V = rng.integers(-3, 4, (m, n)) if dt == np.int32 else rng.standard_normal((m, n))
    from graphs import dense_to_csr
    return dense_to_csr(D, V, dt)


@pytest.mark.parametrize("dt", [np.int32, np.float64])
@pytest.mark.parametrize("shape", [(60, 45), (400, 3000)])
def test_ewise_add_and_mult(ctx, dt, shape):
    rng = np.random.default_rng(shape[0] + (dt == np.float64))
    m, n = shape
    A, B, M = hub_csr(m, n, rng, dt), hub_csr(m, n, rng, dt, 5), hub_csr(m, n, rng, dt, 3)
    dA, dB, dM = (to_device(ctx, X) for X in (A, B, M))
    check(ga.ewise_add(dA, dB), oracle.ewise_add(A, B))
    check(ga.ewise_add(dA, dB, dM), oracle.ewise_add(A, B, M))
    check(ga.ewise_mult(dA, dB), oracle.ewise_mult(A, B))
    check(ga.ewise_mult(dA, dB, dM), oracle.ewise_mult(A, B, M))
    # a shared pattern: values cancel to zero and drop out of the masked sum
    negB = oracle.Csr(A.m, A.n, A.rst, A.col, (-A.val).astype(dt))
    check(ga.ewise_add(dA, to_device(ctx, negB), dM), oracle.ewise_add(A, negB, M))


@pytest.mark.parametrize("dt", [np.int32, np.float64])
def test_mult_scalar(ctx, dt):
    rng = np.random.default_rng(9)
    A = random_csr(80, 70, 0.1, rng, dt)
    dA = to_device(ctx, A)
    ga.mult_scalar(dA, -1.75)
    check(dA, oracle.mult_scalar(A, -1.75))


@pytest.mark.parametrize("dt", [np.int32, np.float64])
def test_mxv_vxm(ctx, dt):
    rng = np.random.default_rng(12)
    m, n = 500, 2000
    A = hub_csr(m, n, rng, dt)
    dA = to_device(ctx, A)
    code = ga.INT32 if dt == np.int32 else ga.FP64
    xn = random_csr(1, n, 1.0, rng, dt).val
    ym = random_csr(1, m, 1.0, rng, dt).val
    x = ga.Dense.create(ctx, n, 1, code, xn)
    y = ga.Dense.create(ctx, m, 1, code, ym)
    ga.mxv(dA, x, y)
    assert np.array_equal(y.download().ravel().view(np.uint8), oracle.mxv(A, xn, ym).view(np.uint8))
    xm = random_csr(1, m, 1.0, rng, dt).val
    yn = random_csr(1, n, 1.0, rng, dt).val
    x2 = ga.Dense.create(ctx, m, 1, code, xm)
    y2 = ga.Dense.create(ctx, 1, n, code, yn)
    ga.vxm(dA, x2, y2)
    assert np.array_equal(y2.download().ravel().view(np.uint8), oracle.vxm(A, xm, yn).view(np.uint8))
    with pytest.raises(ga.GaError) as e:
        ga.mxv(dA, x2, y2)
    assert e.value.code == ga.ERR_SHAPE


def test_ewise_shape_checks(ctx):
    rng = np.random.default_rng(1)
    A = to_device(ctx, random_csr(10, 12, 0.3, rng))
    B = to_device(ctx, random_csr(10, 13, 0.3, rng))
    with pytest.raises(ga.GaError) as e:
        ga.ewise_add(A, B)
    assert e.value.code == ga.ERR_SHAPE
    F = to_device(ctx, random_csr(10, 12, 0.3, rng, np.float64))
    with pytest.raises(ga.GaError) as e:
        ga.ewise_mult(A, F)
    assert e.value.code == ga.ERR_DTYPE
