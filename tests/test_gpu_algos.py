"""Parity of triangle counting, k-truss and batched BC with the CPU oracle.

TC totals, per-row counts and k-truss edge sets are bit-exact; BC scores
(FP64) agree within 1e-9 relative (absolute floor 1e-9).
"""
import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle
from graphs import csr_from_arrays, random_graph, to_device

pytestmark = pytest.mark.gpu

BC_RTOL = 1e-9


def _graphs():
    rng = np.random.default_rng(2024)
    yield "er1000", csr_from_arrays(*ga.gen_er(1000, 9990, seed=7))
    yield "rmat10", csr_from_arrays(*ga.gen_rmat(10, 16, seed=3))
    yield "rmat12", csr_from_arrays(*ga.gen_rmat(12, 16, seed=4))
    yield "knn600", csr_from_arrays(*ga.gen_knn(600, 6, 30, seed=5))
    yield "dense60", random_graph(60, 0.5, rng)
    yield "tiny", random_graph(5, 0.6, rng)


GRAPHS = list(_graphs())


@pytest.mark.parametrize("algo", ["dot", "msa", "mca", "heap", "naive"])
@pytest.mark.parametrize("name,G", GRAPHS, ids=[g[0] for g in GRAPHS])
def test_tc(ctx, algo, name, G):
    if algo == "naive" and G.m > 2000:
        pytest.skip("naive builds the full product")
    total, rows = oracle.tc_sandia(G)
    got, grow = ga.tc(algo, to_device(ctx, G))
    assert got == total
    assert np.array_equal(grow, rows)


def test_tc_other_forms(ctx):
    G = csr_from_arrays(*ga.gen_rmat(9, 16, seed=11))
    total, _ = oracle.tc_sandia(G)
    Gd = to_device(ctx, G)
    assert ga.tc_lu("msa", Gd) == total
    # per-vertex: (A*A<A> row sums) / 2, the reference's int arithmetic
    sq = oracle.mxm_masked(G, G, G)
    ref = np.array([int(sq[G.rst[i]:G.rst[i + 1]].sum()) >> 1 for i in range(G.m)], np.int32)
    assert np.array_equal(ga.tc_vertex("msa", Gd), ref)
    assert int(ref.sum()) == 3 * total


@pytest.mark.parametrize("algo", ["msa", "mca", "heap", "dot", "hybrid"])
@pytest.mark.parametrize("device_loops", [1, 0])
def test_ktruss(ctx, algo, device_loops):
    ctx.set_option(ga.OPT_DEVICE_LOOPS, device_loops)
    try:
        for name, G in GRAPHS[:4]:
            Gd = to_device(ctx, G)
            for k in (3, 4, 5, 7):
                R, it = oracle.ktruss(G, k)
                C, git = ga.ktruss(algo, Gd, k)
                r, c, v = C.download()
                assert git == it, (name, k)
                assert np.array_equal(r, R.rst) and np.array_equal(c, R.col) and np.array_equal(v, R.val), (name, k)
    finally:
        ctx.set_option(ga.OPT_DEVICE_LOOPS, 1)


def test_ktruss_dot_needs_symmetric(ctx):
    rng = np.random.default_rng(4)
    D = np.triu(rng.random((30, 30)) < 0.3, 1)
    from graphs import dense_to_csr
    G = dense_to_csr(D)  # upper triangle only: not symmetric
    with pytest.raises(ga.GaError) as e:
        ga.ktruss("dot", to_device(ctx, G), 3)
    assert e.value.code == ga.ERR_UNSUPPORTED


def test_ktruss_naive_and_trivial_k(ctx):
    G = csr_from_arrays(*ga.gen_knn(300, 4, 30, seed=9))
    Gd = to_device(ctx, G)
    for k in (2, 6):
        R, it = oracle.ktruss(G, k)
        C, git = ga.ktruss("naive", Gd, k)
        r, c, v = C.download()
        assert git == it and np.array_equal(c, R.col) and np.array_equal(v, R.val)


def _bc_close(got, ref):
    err = np.abs(got - ref)
    assert np.all(err <= BC_RTOL * np.maximum(np.abs(ref), 1.0)), float(np.max(err / np.maximum(np.abs(ref), 1.0)))


@pytest.mark.parametrize("device_loops", [1, 0])
def test_bc(ctx, device_loops):
    ctx.set_option(ga.OPT_DEVICE_LOOPS, device_loops)
    try:
        rng = np.random.default_rng(77)
        for name, G in GRAPHS:
            for ns in (1, 7, 64):
                ns = min(ns, G.m)
                src = rng.choice(G.m, ns, replace=False).astype(np.int32)
                ref = oracle.bc_batch(G, src)
                got = ga.bc(to_device(ctx, G), src)
                _bc_close(got, ref)
    finally:
        ctx.set_option(ga.OPT_DEVICE_LOOPS, 1)


def test_bc_directed_and_weighted(ctx):
    rng = np.random.default_rng(78)
    from graphs import dense_to_csr
    D = rng.random((200, 200)) < 0.03
    np.fill_diagonal(D, False)
    G = dense_to_csr(D, rng.integers(1, 3, size=(200, 200)), np.int32)
    src = rng.choice(200, 33, replace=False).astype(np.int32)
    _bc_close(ga.bc(to_device(ctx, G), src), oracle.bc_batch(G, src))


def test_bc_rejects_bad_sources(ctx):
    G = csr_from_arrays(*ga.gen_er(100, 300, seed=1))
    Gd = to_device(ctx, G)
    with pytest.raises(ga.GaError):
        ga.bc(Gd, [1, 1])
    with pytest.raises(ga.GaError):
        ga.bc(Gd, [100])


def test_async_download_overlaps_and_orders_free(ctx):
    """ga_csr_download_async copies on the context's copy stream; a free right
    after it is ordered behind the copy, and the data equal a plain download."""
    import ctypes
    G = csr_from_arrays(*ga.gen_rmat(12, 16, seed=13))
    A = to_device(ctx, G)
    C, _ = ga.ktruss("msa", A, 4)
    ref = C.download()
    rst = np.empty(G.m + 1, np.int32)
    col = np.empty(max(1, C.nnz), np.int32)
    ga.host_register(rst)
    ga.host_register(col)
    try:
        rc = ga.lib().ga_csr_download_async(ctx.handle, C.handle, rst.ctypes.data_as(ctypes.c_void_p),
                                            col.ctypes.data_as(ctypes.c_void_p), None)
        assert rc == ga.OK
        C.free()
        D, _ = ga.ktruss("msa", A, 5)  # new work (and allocations) queued behind the free
        assert ga.lib().ga_ctx_copy_sync(ctx.handle) == ga.OK
        assert np.array_equal(rst, ref[0]) and np.array_equal(col[:len(ref[1])], ref[1])
        D.free()
    finally:
        ga.host_unregister(rst)
        ga.host_unregister(col)
