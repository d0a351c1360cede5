"""Parity of triangle counting, k-truss and batched BC with the CPU oracle.

TC totals, per-row counts and k-truss edge sets are bit-exact; BC scores
(FP64) agree within 1e-9 relative (absolute floor 1e-9).
"""
import os

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


@pytest.mark.parametrize("algo", ["dot", "msa", "mca", "heap", "naive", "tri"])
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
    # triangle listing for the per-vertex form (C<A> = A*A of a symmetric 0/1
    # matrix); the L*U form's operands differ, so GA_TRI runs the hybrid form
    assert np.array_equal(ga.tc_vertex("tri", Gd), ref)
    assert ga.tc_lu("tri", Gd) == total


@pytest.mark.parametrize("algo", ["msa", "mca", "heap", "dot", "hybrid", "tri"])
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


def test_symmetry_check_cases(ctx):
    """The device symmetry check searches the mirror of each entry above the
    diagonal and compares the counts above and below it: a symmetric matrix
    passes (diagonal entries allowed); an extra entry below the diagonal, an
    extra entry above it, or one value that differs from its mirror's makes
    it not symmetric (GA_DOT k-truss refuses it)."""
    rng = np.random.default_rng(12)
    from graphs import dense_to_csr
    D = rng.random((300, 300)) < 0.05
    D = D | D.T
    np.fill_diagonal(D, False)
    D[7, 7] = True
    V = rng.integers(1, 9, size=(300, 300))
    V = np.triu(V) + np.triu(V, 1).T
    i, j = [(a, b) for a, b in zip(*np.nonzero(D)) if a > b][5]
    lower, upper, val = D.copy(), D.copy(), V.copy()
    lower[j, i] = False  # (i, j) below the diagonal loses its mirror
    upper[i, j] = False  # (j, i) above the diagonal loses its mirror
    val[i, j] += 1
    G = dense_to_csr(D, V)
    R, it = oracle.ktruss(G, 3)
    C, git = ga.ktruss("dot", to_device(ctx, G), 3)
    r, c, v = C.download()
    assert git == it and np.array_equal(r, R.rst) and np.array_equal(c, R.col) and np.array_equal(v, R.val)
    for M, W in ((lower, V), (upper, V), (D, val)):
        with pytest.raises(ga.GaError) as e:
            ga.ktruss("dot", to_device(ctx, dense_to_csr(M, W)), 3)
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


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_bc_backward_modes(ctx, mode):
    """GA_OPT_BC_BACKWARD: gathered W rows (0), bulk copies of whole rows
    into shared memory (1; odd source counts and more than 128 sources fall
    back to 0) and one neighbour at a time (2) all match the FP64 oracle; a
    vertex with more than 1,024 neighbours (a CTA-shared row) is included."""
    rng = np.random.default_rng(91)
    from graphs import dense_to_csr
    D = rng.random((300, 300)) < 0.05
    np.fill_diagonal(D, False)
    W = dense_to_csr(D, rng.integers(1, 4, size=(300, 300)), np.int32)
    # a star centre with 1,500 neighbours next to an R-MAT core
    m = 1600
    r = list(range(1, 1501))
    edges = [(0, j) for j in r] + [(j, 0) for j in r]
    er = ga.gen_rmat(9, 8, seed=13)
    rows = np.repeat(np.arange(er[0]), np.diff(er[1])) + 1000
    edges += list(zip(rows.tolist(), (er[2] + 1000).tolist()))
    edges += [(5, 1001), (1001, 5)]
    E = np.array(sorted(set(edges)), dtype=np.int64)
    rst = np.zeros(m + 1, np.int32)
    np.add.at(rst, E[:, 0] + 1, 1)
    S = csr_from_arrays(m, np.cumsum(rst).astype(np.int32), E[:, 1].astype(np.int32))
    ctx.set_option(ga.OPT_BC_BACKWARD, mode)
    try:
        for G, counts in ((S, (64, 33, 130)), (W, (2, 40))):
            for ns in counts:
                src = rng.choice(G.m, ns, replace=False).astype(np.int32)
                _bc_close(ga.bc(to_device(ctx, G), src), oracle.bc_batch(G, src))
    finally:
        ctx.set_option(ga.OPT_BC_BACKWARD, 0)
    with pytest.raises(ga.GaError):
        ctx.set_option(ga.OPT_BC_BACKWARD, 3)


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


def _with_loops(G, rows):
    """G plus diagonal entries (i, i) for the given rows (values 1)."""
    D = np.zeros((G.m, G.m), bool)
    for i in range(G.m):
        D[i, G.col[G.rst[i]:G.rst[i + 1]]] = True
    D[rows, rows] = True
    from graphs import dense_to_csr
    return dense_to_csr(D)


def _tri_graphs():
    rng = np.random.default_rng(99)
    yield from GRAPHS
    # oriented lists longer than 32 (bucket search) and hubs next to leaves
    yield "dense300", random_graph(300, 0.5, rng)
    star = random_graph(400, 0.02, rng)
    D = np.zeros((400, 400), bool)
    for i in range(400):
        D[i, star.col[star.rst[i]:star.rst[i + 1]]] = True
    D[0, 1:] = D[1:, 0] = True
    D[1, 2:200] = D[2:200, 1] = True
    from graphs import dense_to_csr
    yield "hubs400", dense_to_csr(D)
    yield "loops", _with_loops(random_graph(80, 0.2, rng), rng.choice(80, 25, replace=False))


TRI_GRAPHS = list(_tri_graphs())


def test_tri_support_wide_rank_spans(ctx):
    """Lists whose ranks span more than the 16,384-rank window (a graph of
    40,000 vertices where every vertex links to random far vertices and to
    a few hubs): members below the window are found by the binary search."""
    rng = np.random.default_rng(31)
    n = 40000
    src = rng.integers(0, n, 200000)
    dst = rng.integers(0, n, 200000)
    hubs = rng.choice(n, 20, replace=False)
    src = np.concatenate([src, np.repeat(hubs, 3000)])
    dst = np.concatenate([dst, rng.integers(0, n, 60000)])
    keep = src != dst
    a, b = np.concatenate([src[keep], dst[keep]]), np.concatenate([dst[keep], src[keep]])
    key = np.unique(a.astype(np.int64) * n + b)
    r, c = (key // n).astype(np.int32), (key % n).astype(np.int32)
    rst = np.zeros(n + 1, np.int32)
    np.add.at(rst, r + 1, 1)
    G = csr_from_arrays(n, np.cumsum(rst).astype(np.int32), c)
    ref = oracle.mxm_masked(G, G, G)
    Gd = to_device(ctx, G)
    for order in (0, 1):
        ctx.set_option(ga.OPT_TRI_ORDER, order)
        try:
            _, _, v = ga.mxm_masked("tri", Gd, Gd, Gd).download()
            assert np.array_equal(v, np.asarray(ref, np.int32)), order
            assert ga.tc("tri", Gd)[0] == oracle.tc_sandia(G)[0]
        finally:
            ctx.set_option(ga.OPT_TRI_ORDER, 0)


@pytest.mark.parametrize("name,G", TRI_GRAPHS, ids=[g[0] for g in TRI_GRAPHS])
def test_tri_support_product(ctx, name, G):
    """C<A> = A*A by triangle listing equals the Gustavson product bit for bit
    (diagonal entries included), and the wedge / triangle counters agree with
    a count of the triangles."""
    ref = oracle.mxm_masked(G, G, G)
    Gd = to_device(ctx, G)
    ctx.work_counters(reset=True)
    C = ga.mxm_masked("tri", Gd, Gd, Gd)
    wt = ctx.work_counters(reset=True)
    _, c, v = C.download()
    assert np.array_equal(c, G.col) and np.array_equal(v, np.asarray(ref, np.int32))
    # the same Gustavson work figures as the MSA form reports
    ga.mxm_masked("msa", Gd, Gd, Gd)
    wm = ctx.work_counters(reset=True)
    assert wt["products"] == wm["products"] and wt["mask_entries"] == wm["mask_entries"]
    loops = any(i in G.col[G.rst[i]:G.rst[i + 1]] for i in range(G.m))
    if not loops:
        assert wt["triangles"] == oracle.tc_sandia(G)[0]


@pytest.mark.parametrize("device_loops,order", [(1, 0), (0, 0), (1, 1)])
def test_tri_ktruss_with_loops_and_hubs(ctx, device_loops, order):
    ctx.set_option(ga.OPT_DEVICE_LOOPS, device_loops)
    ctx.set_option(ga.OPT_TRI_ORDER, order)
    try:
        for name, G in TRI_GRAPHS[-3:]:
            Gd = to_device(ctx, G)
            for k in (3, 4, 6, 9):
                R, it = oracle.ktruss(G, k)
                C, git = ga.ktruss("tri", Gd, k)
                r, c, v = C.download()
                assert git == it, (name, k)
                assert np.array_equal(r, R.rst) and np.array_equal(c, R.col) and np.array_equal(v, R.val), (name, k)
    finally:
        ctx.set_option(ga.OPT_DEVICE_LOOPS, 1)
        ctx.set_option(ga.OPT_TRI_ORDER, 0)


def test_tri_falls_back_for_other_operands(ctx):
    """Operands GA_TRI does not cover (different matrices, non-unit values,
    a non-symmetric matrix) get the hybrid form's results."""
    rng = np.random.default_rng(5)
    from graphs import random_csr
    A = random_csr(50, 60, 0.2, rng)
    B = random_csr(60, 40, 0.2, rng)
    M = random_csr(50, 40, 0.3, rng)
    ref = oracle.mxm_masked(A, B, M)
    _, _, v = ga.mxm_masked("tri", to_device(ctx, A), to_device(ctx, B), to_device(ctx, M)).download()
    assert np.array_equal(v, np.asarray(ref, np.int32))
    G = random_graph(70, 0.2, rng)
    W = oracle.Csr(G.m, G.n, G.rst, G.col, np.full(G.nnz, 2, np.int32))  # symmetric, values 2
    Wd = to_device(ctx, W)
    _, _, v = ga.mxm_masked("tri", Wd, Wd, Wd).download()
    assert np.array_equal(v, np.asarray(oracle.mxm_masked(W, W, W), np.int32))
    for k in (3, 5):
        R, it = oracle.ktruss(W, k)
        C, git = ga.ktruss("tri", Wd, k)
        r, c, vv = C.download()
        assert git == it and np.array_equal(c, R.col) and np.array_equal(vv, R.val)


@pytest.mark.parametrize("name,G", TRI_GRAPHS[-3:], ids=[g[0] for g in TRI_GRAPHS[-3:]])
def test_tri_tc_long_lists_and_loops(ctx, name, G):
    """Triangle listing counts like the Sandia form (diagonal entries ignored,
    per-row counts = triangles whose largest vertex is the row); a matrix
    that is not symmetric takes the Sandia form."""
    total, rows = oracle.tc_sandia(G)
    got, grow = ga.tc("tri", to_device(ctx, G))
    assert got == total and np.array_equal(grow, rows)
    rng = np.random.default_rng(12)
    from graphs import dense_to_csr
    D = rng.random((90, 90)) < 0.15
    np.fill_diagonal(D, False)
    N = dense_to_csr(D)  # not symmetric
    total, rows = oracle.tc_sandia(N)
    got, grow = ga.tc("tri", to_device(ctx, N))
    assert got == total and np.array_equal(grow, rows)


def test_tri_ktruss_degenerate_inputs(ctx):
    """k <= 2 keeps everything; graphs without entries, with diagonal entries
    only, or without vertices, as the oracle has them."""
    from graphs import dense_to_csr
    rng = np.random.default_rng(17)
    G = random_graph(40, 0.2, rng)
    cases = [(G, k) for k in (1, 2)]
    cases.append((dense_to_csr(np.zeros((30, 30), bool)), 3))           # no entries
    cases.append((dense_to_csr(np.eye(25, dtype=bool)), 3))              # diagonal only
    cases.append((dense_to_csr(np.eye(25, dtype=bool)), 4))
    for H, k in cases:
        R, it = oracle.ktruss(H, k)
        C, git = ga.ktruss("tri", to_device(ctx, H), k)
        r, c, v = C.download()
        assert git == it and np.array_equal(r, R.rst) and np.array_equal(c, R.col), (H.m, H.nnz, k)
        assert np.array_equal(v, R.val)
        assert ga.tc("tri", to_device(ctx, H))[0] == oracle.tc_sandia(H)[0]
    E = ga.Csr.upload(ctx, 0, 0, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32))
    C, git = ga.ktruss("tri", E, 3)
    assert C.nnz == 0 and git == 0


@pytest.mark.parametrize("algo", ["tri", "hybrid"])
def test_ktruss_full_sweep_rmat16(ctx, algo):
    """The benchmark's sweep on a smaller R-MAT graph (scale 16, edge factor
    16): C_3 = k_truss(A, 3), then C_k = k_truss(C_{k-1}, k) until the truss
    is empty; every k-truss (edge set, values, iteration count) equals the
    oracle's, and the device sweep ends at the oracle's k_max."""
    m, rst, col = ga.gen_rmat(16, 16, 0.57, 0.19, 0.19, seed=42)
    cur_h = csr_from_arrays(m, rst, col)
    cur_d = ga.Csr.upload(ctx, m, m, rst, col, np.ones(len(col), np.int32))
    k = 3
    while True:
        R, it = oracle.ktruss(cur_h, k)
        C, git = ga.ktruss(algo, cur_d, k)
        r, c, v = C.download()
        assert git == it, k
        assert np.array_equal(r, R.rst) and np.array_equal(c, R.col) and np.array_equal(v, R.val), k
        cur_d.free()
        cur_h, cur_d = R, C
        if R.nnz == 0:
            break
        k += 1
    assert k > 20  # a power-law graph: a long sweep


@pytest.mark.parametrize("algo", ["tri", "msa"])
@pytest.mark.parametrize("device_loops", [1, 0])
def test_ktruss_sweep_api(ctx, algo, device_loops):
    """ga_ktruss_sweep (with triangle listing one device-resident state for
    the whole sweep; otherwise one ga_ktruss per k) against the oracle run
    stage by stage on R-MAT 14: every k-truss (edge set, values, iteration
    count) equal, the same k_max, and the same Gustavson-product count as the
    stage-by-stage ga_ktruss calls. A sweep can start at k <= 2 (nothing
    pruned) and on a matrix without entries."""
    ctx.set_option(ga.OPT_DEVICE_LOOPS, device_loops)
    try:
        m, rst, col = ga.gen_rmat(14, 16, 0.57, 0.19, 0.19, seed=5)
        A = ga.Csr.upload(ctx, m, m, rst, col, np.ones(len(col), np.int32))
        cur_h = csr_from_arrays(m, rst, col)
        ctx.work_counters(reset=True)
        got = []
        for k, C, it in ga.ktruss_sweep(algo, A, 2):
            r, c, v = C.download()
            C.free()
            got.append((k, it, r, c, v))
        products_sweep = ctx.work_counters(reset=True)["products"]
        ks = [g[0] for g in got]
        assert ks == list(range(2, 2 + len(got))) and len(got) > 10
        for k, it, r, c, v in got:
            R, rit = oracle.ktruss(cur_h, k)
            assert it == rit, k
            assert np.array_equal(r, R.rst) and np.array_equal(c, R.col) and np.array_equal(v, R.val), k
            cur_h = R
        assert got[-1][2][-1] == 0 and all(g[2][-1] > 0 for g in got[:-1])
        # the same work counted as the stage-by-stage calls
        cur = A
        for k in ks:
            C, _ = ga.ktruss(algo, cur, k)
            if cur is not A:
                cur.free()
            cur = C
        cur.free()
        assert ctx.work_counters(reset=True)["products"] == products_sweep
        # diagonal entries: a diagonal entry's support is its row's length
        rng = np.random.default_rng(4)
        from graphs import dense_to_csr
        U = np.triu(rng.random((80, 80)) < 0.3, 1)
        D = U | U.T
        D[np.arange(0, 80, 3), np.arange(0, 80, 3)] = True
        G = dense_to_csr(D)
        cur_h = G
        for k, C, it in ga.ktruss_sweep(algo, to_device(ctx, G), 3):
            R, rit = oracle.ktruss(cur_h, k)
            r, c, _ = C.download()
            assert it == rit and np.array_equal(r, R.rst) and np.array_equal(c, R.col), k
            cur_h = R
        assert cur_h.nnz == 0
        E = ga.Csr.upload(ctx, 5, 5, np.zeros(6, np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32))
        out = [(k, C.nnz, it) for k, C, it in ga.ktruss_sweep(algo, E, 3)]
        C0, it0 = ga.ktruss(algo, E, 3)
        assert out == [(3, 0, it0)], out
    finally:
        ctx.set_option(ga.OPT_DEVICE_LOOPS, 1)


@pytest.mark.parametrize("device_loops", [1, 0])
def test_tri_ktruss_frontier_equals_relisting(ctx, device_loops):
    """The frontier form of the GA_TRI k-truss (one listing, then only the
    triangles of the pruned edges) against the form that lists every triangle
    in every iteration: the same edge sets and iteration counts, and the same
    Gustavson-product, mask-entry and entry counters (the reference's work,
    counted per iteration)."""
    ctx.set_option(ga.OPT_DEVICE_LOOPS, device_loops)
    graphs = [(n, G) for n, G in TRI_GRAPHS] + [("rmat14", csr_from_arrays(*ga.gen_rmat(14, 16, seed=8)))]
    try:
        for name, G in graphs:
            Gd = to_device(ctx, G)
            for k in (3, 4, 5, 8, 12):
                out = []
                for frontier in (1, 0):
                    ctx.set_option(ga.OPT_KT_FRONTIER, frontier)
                    ctx.work_counters(reset=True)
                    C, it = ga.ktruss("tri", Gd, k)
                    wc = ctx.work_counters(reset=True)
                    out.append((it, C.download(), {x: wc[x] for x in ("products", "mask_entries", "a_entries",
                                                                      "launches", "rows")}))
                    C.free()
                (it1, (r1, c1, v1), w1), (it0, (r0, c0, v0), w0) = out
                assert it1 == it0, (name, k)
                assert np.array_equal(r1, r0) and np.array_equal(c1, c0) and np.array_equal(v1, v0), (name, k)
                assert w1 == w0, (name, k, w1, w0)
    finally:
        ctx.set_option(ga.OPT_KT_FRONTIER, 1)
        ctx.set_option(ga.OPT_DEVICE_LOOPS, 1)


def test_bc_all_sources(ctx):
    """All-source BC (betweenness_centrality.h:5-123) accumulated on the
    device, against the FP64 oracle's blocked form, 1e-9 relative: ragged
    last blocks, blocks of one source, blocks above one device batch (1,024
    sources) and above m; a directed weighted graph; block 0 refused."""
    rng = np.random.default_rng(91)
    G = csr_from_arrays(*ga.gen_rmat(10, 8, seed=21))
    Gd = to_device(ctx, G)
    ref = oracle.bc_all(G, 100)
    for block in (100, 64, 1, 1500, 5000):
        _bc_close(ga.bc_all(Gd, block), ref)
    from graphs import dense_to_csr
    D = rng.random((150, 150)) < 0.04
    np.fill_diagonal(D, False)
    W = dense_to_csr(D, rng.integers(1, 3, size=(150, 150)), np.int32)
    _bc_close(ga.bc_all(to_device(ctx, W), 33), oracle.bc_all(W, 33))
    with pytest.raises(ga.GaError) as e:
        ga.bc_all(Gd, 0)
    assert e.value.code == ga.ERR_INVALID_ARG


def test_declared_symmetry(ctx):
    """ga_csr_set_symmetric: a symmetric graph declared symmetric skips the
    device check and gives the same results; declared not symmetric, the
    k-truss and BC take their general forms (same results); -1 checks
    again; a non-square matrix cannot be declared symmetric."""
    G = csr_from_arrays(*ga.gen_rmat(11, 16, seed=19))
    R, it = oracle.ktruss(G, 5)
    src = np.arange(0, 40, dtype=np.int32)
    ref_bc = oracle.bc_batch(G, src)
    for decl in (1, 0, -1):
        Gd = to_device(ctx, G)
        Gd.set_symmetric(decl)
        C, git = ga.ktruss("tri", Gd, 5)
        r, c, _ = C.download()
        assert git == it and np.array_equal(r, R.rst) and np.array_equal(c, R.col), decl
        _bc_close(ga.bc(Gd, src), ref_bc)
    N = ga.Csr.upload(ctx, 3, 4, np.array([0, 1, 1, 1], np.int32), np.array([2], np.int32))
    with pytest.raises(ga.GaError) as e:
        N.set_symmetric(1)
    assert e.value.code == ga.ERR_SHAPE


def test_ktruss_sweep_rmat18_matches_oracle_record(ctx):
    """The benchmark's own workload through ga_ktruss_sweep: R-MAT scale 18
    (edge factor 16, seed 42), k = 3 ... until empty; every k-truss's
    iteration count, entry count and BLAKE2b digest of (row starts, columns)
    equal the oracle's record of the same sweep (tests/golden/rmat18_sweep.json,
    made by tests/golden/make_sweep.py), and the sweep ends where it ends."""
    import hashlib
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rmat18_sweep.json")
    with open(path) as f:
        rec = json.load(f)
    g = rec["graph"]
    m, rst, col = ga.gen_rmat(g["scale"], g["edge_factor"], *g["abc"], seed=g["seed"])
    assert m == g["vertices"] and len(col) == g["stored_entries"]

    def digest(r, c):
        h = hashlib.blake2b(digest_size=16)
        h.update(np.ascontiguousarray(r, "<i4").tobytes())
        h.update(np.ascontiguousarray(c, "<i4").tobytes())
        return h.hexdigest()

    assert digest(rst, col) == g["digest"]
    A = ga.Csr.upload(ctx, m, m, rst, col)
    got = []
    for k, C, it in ga.ktruss_sweep("tri", A, 3):
        z = C.nnz
        r, c, _ = C.download()
        C.free()
        got.append([k, it, z, digest(r, c[:z])])
    assert got == [list(s) for s in rec["stages"]]


def test_bc_rmat20_64_sources_against_oracle(ctx):
    """Config 3 at its full size: batched BC on R-MAT scale 20 (edge factor
    16, seed 42) with 64 seeded sources, every score within 1e-9 relative of
    the FP64 oracle (OpenMP on the host cores), in all three forms of the
    backward sweep."""
    m, rst, col = ga.gen_rmat(20, 16, 0.57, 0.19, 0.19, seed=42)
    G = csr_from_arrays(m, rst, col)
    src = np.random.default_rng(42).choice(m, 64, replace=False).astype(np.int32)
    oracle.set_num_threads(os.cpu_count() or 1)
    ref = oracle.bc_batch(G, src)
    A = ga.Csr.upload(ctx, m, m, rst, col)
    A.set_symmetric(1)
    try:
        for mode in (0, 1, 2):
            ctx.set_option(ga.OPT_BC_BACKWARD, mode)
            _bc_close(ga.bc(A, src), ref)
    finally:
        ctx.set_option(ga.OPT_BC_BACKWARD, 0)
