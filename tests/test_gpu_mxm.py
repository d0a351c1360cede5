"""Parity of the CUDA masked-SpGEMM family with the CPU oracle.

Integer results must be bit-exact; floating-point values (summation order on
the GPU is not fixed) must agree within rtol 1e-12 (FP64) / 1e-5 (FP32)
relative to the sum of |products|.
"""
import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle
from graphs import random_csr, random_graph, to_device

pytestmark = pytest.mark.gpu

ALGOS = ["msa", "mca", "heap", "naive", "dot", "hybrid"]


def _abs_product(A, B, M):
    Aa = oracle.Csr(A.m, A.n, A.rst, A.col, np.abs(A.val).astype(np.float64))
    Ba = oracle.Csr(B.m, B.n, B.rst, B.col, np.abs(B.val).astype(np.float64))
    return oracle.mxm_masked(Aa, Ba, M)


def _check_vals(got, ref, A, B, M, dtype):
    if np.dtype(dtype).kind in "iu":
        assert np.array_equal(got, ref)
    else:
        scale = _abs_product(A, B, M) + 1e-300
        tol = 1e-12 if np.dtype(dtype) == np.float64 else 1e-5
        assert np.all(np.abs(got.astype(np.float64) - ref.astype(np.float64)) <= tol * scale + 1e-30)


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("dtype", [np.int32, np.int64, np.float32, np.float64])
def test_masked_random(ctx, algo, dtype):
    rng = np.random.default_rng(11)
    for trial in range(6):
        m = int(rng.integers(1, 90))
        k = int(rng.integers(1, 90))
        n = int(rng.integers(1, 90))
        A = random_csr(m, k, rng.random() * 0.3, rng, dtype)
        B = random_csr(k, n, rng.random() * 0.3, rng, dtype)
        M = random_csr(m, n, rng.random() * 0.6, rng, dtype)
        ref = oracle.mxm_masked(A, B, M)
        C = ga.mxm_masked(algo, to_device(ctx, A), to_device(ctx, B), to_device(ctx, M))
        rst, col, val = C.download()
        assert np.array_equal(rst, M.rst) and np.array_equal(col, M.col)
        _check_vals(val, ref, A, B, M, dtype)


@pytest.mark.parametrize("algo", ["msa", "mca", "heap", "dot", "hybrid"])
def test_masked_uint8_wraps_like_reference(ctx, algo):
    rng = np.random.default_rng(3)
    A = random_csr(70, 70, 0.5, rng, np.uint8)
    M = random_csr(70, 70, 0.5, rng, np.uint8)
    A32 = oracle.Csr(A.m, A.n, A.rst, A.col, A.val.astype(np.int32))
    M32 = oracle.Csr(M.m, M.n, M.rst, M.col, M.val.astype(np.int32))
    ref = (oracle.mxm_masked(A32, A32, M32) & 0xFF).astype(np.uint8)
    C = ga.mxm_masked(algo, to_device(ctx, A), to_device(ctx, A), to_device(ctx, M))
    assert np.array_equal(C.download()[2], ref)


@pytest.mark.parametrize("algo", ["msa", "mca", "heap", "dot", "hybrid"])
def test_masked_long_rows_and_hubs(ctx, algo):
    """Mask rows longer than one CTA item (4096 slots) and hub rows of B."""
    rng = np.random.default_rng(5)
    n = 9000
    m = 40
    rows_a, rows_m = [], []
    for i in range(m):
        rows_a.append(np.sort(rng.choice(n, size=int(rng.integers(0, 60)), replace=False)))
        sz = 8500 if i % 7 == 0 else int(rng.integers(0, 300))
        rows_m.append(np.sort(rng.choice(n, size=sz, replace=False)))
    def mk(rows, ncols):
        rst = np.zeros(len(rows) + 1, np.int32)
        rst[1:] = np.cumsum([len(r) for r in rows])
        col = np.concatenate(rows).astype(np.int32) if rows else np.zeros(0, np.int32)
        return oracle.Csr(len(rows), ncols, rst, col, np.ones(len(col), np.int32))
    A = mk(rows_a, n)
    brows = []
    for k in range(n):
        sz = 6000 if k % 997 == 0 else int(rng.integers(0, 12))
        brows.append(np.sort(rng.choice(n, size=sz, replace=False)))
    B = mk(brows, n)
    B = oracle.Csr(B.m, B.n, B.rst, B.col, rng.integers(1, 5, len(B.col)).astype(np.int32))
    M = mk(rows_m, n)
    ref = oracle.mxm_masked(A, B, M)
    C = ga.mxm_masked(algo, to_device(ctx, A), to_device(ctx, B), to_device(ctx, M))
    assert np.array_equal(C.download()[2], ref)


def test_masked_support_rmat18_all_variants(ctx):
    """The bench's support product C<A> = A*A on R-MAT 18 (edge factor 16,
    seed 42: rows of up to 25,000 entries, so CTA items over several windows,
    hub B rows and warp rows all occur), with unit values and with values
    1..3: every variant equal to the oracle."""
    m, rst, col = ga.gen_rmat(18, 16, seed=42)
    rng = np.random.default_rng(18)
    for vals in (np.ones(len(col), np.int32), rng.integers(1, 4, len(col)).astype(np.int32)):
        A = oracle.Csr(m, m, rst, col, vals)
        ref = oracle.mxm_masked(A, A, A)
        Ad = to_device(ctx, A)
        algos = ["msa", "mca", "heap", "dot", "hybrid"] + (["tri"] if vals[0] == 1 and np.all(vals == 1) else [])
        for algo in algos:
            C = ga.mxm_masked(algo, Ad, Ad, Ad)
            assert np.array_equal(C.download()[2], ref), algo
            C.free()


@pytest.mark.parametrize("algo", ALGOS)
def test_masked_square_graphs(ctx, algo):
    rng = np.random.default_rng(21)
    for n, d in [(1, 0.0), (5, 0.5), (64, 0.1), (300, 0.05), (600, 0.3)]:
        G = random_graph(n, d, rng)
        ref = oracle.mxm_masked(G, G, G)
        Gd = to_device(ctx, G)
        C = ga.mxm_masked(algo, Gd, Gd, Gd)
        assert np.array_equal(C.download()[2], ref)


def test_masked_empty_inputs(ctx):
    E = oracle.Csr(4, 4, np.zeros(5, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32))
    rng = np.random.default_rng(0)
    A = random_csr(4, 4, 0.6, rng)
    for algo in ALGOS:
        C = ga.mxm_masked(algo, to_device(ctx, A), to_device(ctx, A), to_device(ctx, E))
        assert C.nnz == 0
        C = ga.mxm_masked(algo, to_device(ctx, E), to_device(ctx, A), to_device(ctx, A))
        assert np.array_equal(C.download()[2], np.zeros(A.nnz, np.int32))


@pytest.mark.parametrize("dtype", [np.int32, np.float64])
def test_cmask_random(ctx, dtype):
    rng = np.random.default_rng(8)
    for trial in range(8):
        m = int(rng.integers(1, 80))
        k = int(rng.integers(1, 80))
        n = int(rng.integers(1, 80))
        A = random_csr(m, k, rng.random() * 0.4, rng, dtype)
        B = random_csr(k, n, rng.random() * 0.4, rng, dtype)
        M = random_csr(m, n, rng.random() * 0.5, rng, dtype)
        R = oracle.mxm_cmask(A, B, M)
        C = ga.mxm_cmask(to_device(ctx, A), to_device(ctx, B), to_device(ctx, M))
        rst, col, val = C.download()
        assert np.array_equal(rst, R.rst) and np.array_equal(col, R.col)
        if dtype == np.int32:
            assert np.array_equal(val, R.val)
        else:
            assert np.allclose(val, R.val, rtol=1e-12, atol=1e-12)


def test_cmask_long_rows_use_windows(ctx):
    """Rows with more than 2048 products go through the windowed dense path."""
    rng = np.random.default_rng(9)
    A = random_csr(50, 400, 0.2, rng)
    B = random_csr(400, 9000, 0.05, rng)
    M = random_csr(50, 9000, 0.3, rng)
    R = oracle.mxm_cmask(A, B, M)
    C = ga.mxm_cmask(to_device(ctx, A), to_device(ctx, B), to_device(ctx, M))
    rst, col, val = C.download()
    assert np.array_equal(rst, R.rst) and np.array_equal(col, R.col) and np.array_equal(val, R.val)


def test_cmask_union_is_full_product(ctx):
    """C<!M> plus C<M> (nonzero part) equals the unmasked product."""
    rng = np.random.default_rng(10)
    A = random_csr(60, 60, 0.1, rng)
    M = random_csr(60, 60, 0.2, rng)
    E = oracle.Csr(60, 60, np.zeros(61, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32))
    full = ga.mxm_cmask(to_device(ctx, A), to_device(ctx, A), to_device(ctx, E))
    comp = ga.mxm_cmask(to_device(ctx, A), to_device(ctx, A), to_device(ctx, M))
    fr, fc, fv = full.download()
    cr, cc, cv = comp.download()
    mv = ga.mxm_masked("msa", to_device(ctx, A), to_device(ctx, A), to_device(ctx, M)).download()[2]
    D = np.zeros((60, 60), np.int64)
    for i in range(60):
        D[i, cc[cr[i]:cr[i + 1]]] += cv[cr[i]:cr[i + 1]]
        D[i, M.col[M.rst[i]:M.rst[i + 1]]] += mv[M.rst[i]:M.rst[i + 1]]
    F = np.zeros((60, 60), np.int64)
    for i in range(60):
        F[i, fc[fr[i]:fr[i + 1]]] = fv[fr[i]:fr[i + 1]]
    assert np.array_equal(D, F)


def test_spd_ewise_and_union(ctx):
    rng = np.random.default_rng(12)
    m, ns = 70, 9
    A = random_csr(m, m, 0.1, rng, np.float64)
    Bd = rng.standard_normal((m, ns))
    M = random_csr(m, ns, 0.4, rng, np.float64)
    ref = oracle.mxm_spd(A, Bd, M)
    Bdev = ga.Dense.create(ctx, m, ns, ga.FP64, Bd)
    Cdev = ga.Dense.create(ctx, m, ns, ga.FP64)
    ga.mxm_spd(to_device(ctx, A), Bdev, to_device(ctx, M), Cdev)
    assert np.array_equal(Cdev.download(), ref)  # same summation order: bit-exact
    X = rng.standard_normal((m, ns))
    Y = rng.standard_normal((m, ns))
    Xd, Yd = ga.Dense.create(ctx, m, ns, ga.FP64, X), ga.Dense.create(ctx, m, ns, ga.FP64, Y)
    Zd = ga.Dense.create(ctx, m, ns, ga.FP64)
    ga.ewise_mult_masked(Xd, Yd, to_device(ctx, M), Zd)
    assert np.array_equal(Zd.download(), oracle.ewise_mult_masked(X, Y, M))
    Z0 = rng.standard_normal((m, ns))
    Zd = ga.Dense.create(ctx, m, ns, ga.FP64, Z0)
    ga.fuse_ewise_mult_add(Xd, Yd, Zd)
    assert np.array_equal(Zd.download(), oracle.fuse_ewise_mult_add(X, Y, Z0))
    # add_nointersect on disjoint patterns
    P = rng.random((m, ns)) < 0.3
    Q = (rng.random((m, ns)) < 0.3) & ~P
    from graphs import dense_to_csr
    Pc = dense_to_csr(P, rng.standard_normal((m, ns)), np.float64)
    Qc = dense_to_csr(Q, rng.standard_normal((m, ns)), np.float64)
    R = oracle.add_nointersect(Pc, Qc)
    U = ga.add_nointersect(to_device(ctx, Pc), to_device(ctx, Qc))
    r, c, v = U.download()
    assert np.array_equal(r, R.rst) and np.array_equal(c, R.col) and np.array_equal(v, R.val)


def test_graph_prep(ctx):
    rng = np.random.default_rng(13)
    for n in [1, 7, 120, 500]:
        A = random_csr(n, n, 0.08, rng)
        Ad = to_device(ctx, A)
        for got, ref in [(ga.transpose(Ad), oracle.transpose(A)), (ga.extract_lower(Ad), oracle.extract_lower(A)),
                         (ga.extract_upper(Ad), oracle.extract_upper(A))]:
            r, c, v = got.download()
            assert np.array_equal(r, ref.rst) and np.array_equal(c, ref.col) and np.array_equal(v, ref.val)
        L = oracle.extract_lower(A)
        S = ga.symm_from_lower(to_device(ctx, L))
        ref = oracle.symm_from_lower(L)
        r, c, v = S.download()
        assert np.array_equal(r, ref.rst) and np.array_equal(c, ref.col) and np.array_equal(v, ref.val)


def test_invalid_csr_rejected(ctx):
    with pytest.raises(ga.GaError) as e:
        ga.Csr.upload(ctx, 2, 3, [0, 2, 3], [1, 0, 2])  # row 0 unsorted
    assert e.value.code == ga.ERR_INVALID_CSR
    with pytest.raises(ga.GaError) as e:
        ga.Csr.upload(ctx, 2, 3, [0, 1, 2], [0, 5])  # column out of range
    assert e.value.code == ga.ERR_INVALID_CSR
    with pytest.raises(ga.GaError) as e:
        ga.Csr.upload(ctx, 2, 3, [0, 2, 1], [0, 1])  # row starts not monotone
    assert e.value.code == ga.ERR_INVALID_CSR
