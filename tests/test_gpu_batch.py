"""Batched graphs: a block-diagonal union run by one launch of each kernel
gives every graph the result it gets alone.

Triangle counts, k-truss edge sets and k-truss iteration counts are compared
bit-exactly with per-graph single calls and, for a few graphs, with the
oracle. The device k-NN generator is checked for the structure it promises.
"""
import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle
from graphs import csr_from_arrays, random_graph, to_device

pytestmark = pytest.mark.gpu


def _uneven_sizes(count, lo, hi, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(lo, hi + 1, count).astype(np.int32), rng.integers(4, 17, count).astype(np.int32)


def _check_knn_structure(m, rst, col, k):
    assert rst[0] == 0 and np.all(np.diff(rst) >= 0)
    for i in range(m):
        row = col[rst[i]:rst[i + 1]]
        assert np.all(np.diff(row) > 0), "rows sorted, no duplicates"
        assert not np.any(row == i), "no self-loops"
        assert len(row) >= min(k, m - 1)
    # symmetric pattern
    rows = np.repeat(np.arange(m), np.diff(rst))
    a = set(zip(rows.tolist(), col.tolist()))
    assert all((j, i) in a for i, j in a)


def test_knn_batch_structure(ctx):
    n, dim = _uneven_sizes(12, 1, 300, seed=3)
    n[0], n[1] = 1, 31  # a single point; fewer points than k + 1
    U, voff = ga.gen_knn_batch(ctx, n, dim, k=30, seed=9)
    assert voff[0] == 0 and np.array_equal(np.diff(voff), n)
    rst, col, val = U.download()
    assert np.all(val == 1)
    for g, (m, r, c) in enumerate(ga.split_blocks(rst, col, voff)):
        assert m == n[g]
        assert np.all((c >= 0) & (c < m)), "no edge leaves its graph"
        _check_knn_structure(m, r, c, 30)
    # same seed, same graphs; another seed, other graphs
    U2, _ = ga.gen_knn_batch(ctx, n, dim, k=30, seed=9)
    assert all(np.array_equal(x, y) for x, y in zip(U2.download(), (rst, col, val)))
    U3, _ = ga.gen_knn_batch(ctx, n, dim, k=30, seed=10)
    assert not np.array_equal(U3.download()[1], col)


def _mixed_parts(ctx):
    rng = np.random.default_rng(77)
    host = [
        csr_from_arrays(*ga.gen_er(200, 1500, seed=2)),
        random_graph(1, 0.5, rng),
        csr_from_arrays(*ga.gen_rmat(9, 16, seed=5)),
        random_graph(40, 0.6, rng),
        csr_from_arrays(*ga.gen_knn(300, 5, 30, seed=6)),
        random_graph(3, 0.0, rng),
        random_graph(120, 0.2, rng),
    ]
    return host, [to_device(ctx, G) for G in host]


def test_block_diag_round_trip(ctx):
    host, dev = _mixed_parts(ctx)
    U, voff = ga.block_diag(ctx, dev)
    assert np.array_equal(np.diff(voff), [G.m for G in host])
    rst, col, val = U.download()
    for G, (m, r, c) in zip(host, ga.split_blocks(rst, col, voff)):
        assert m == G.m and np.array_equal(r, G.rst) and np.array_equal(c, G.col)


@pytest.mark.parametrize("algo", ["dot", "msa", "mca", "heap"])
def test_batch_tc_matches_single(ctx, algo):
    host, dev = _mixed_parts(ctx)
    U, voff = ga.block_diag(ctx, dev)
    got = ga.batch_tc(algo, U, voff)
    for g, (G, Gd) in enumerate(zip(host, dev)):
        assert got[g] == ga.tc(algo, Gd, per_row=False)[0]
        assert got[g] == oracle.tc_sandia(G)[0]


def _solo_ktruss(ctx, algo, blocks, k):
    out = []
    for m, r, c in blocks:
        G = ga.Csr.upload(ctx, m, m, r, c, np.ones(len(c), np.int32))
        C, it = ga.ktruss(algo, G, k)
        cr, cc, _ = C.download()
        out.append((cr, cc, it))
    return out


@pytest.mark.parametrize("algo", ["msa", "mca", "heap", "dot", "hybrid", "tri"])
@pytest.mark.parametrize("k", [4, 6])
def test_batch_ktruss_matches_single(ctx, algo, k):
    host, dev = _mixed_parts(ctx)
    U, voff = ga.block_diag(ctx, dev)
    C, iters = ga.batch_ktruss(algo, U, voff, k)
    cr, cc, cv = C.download()
    assert np.all(cv == 1)
    blocks = [(G.m, G.rst, G.col) for G in host]
    for g, ((m, r, c), (sr, sc, sit)) in enumerate(zip(ga.split_blocks(cr, cc, voff),
                                                      _solo_ktruss(ctx, algo, blocks, k))):
        assert iters[g] == sit, f"graph {g}"
        assert np.array_equal(r, sr) and np.array_equal(c, sc), f"graph {g}"
    # two graphs against the oracle as well
    for g in (0, 4):
        ref = oracle.ktruss(host[g], k)
        m, r, c = ga.split_blocks(cr, cc, voff)[g]
        assert np.array_equal(r, ref[0].rst) and np.array_equal(c, ref[0].col)
        assert iters[g] == ref[1]


@pytest.mark.parametrize("device_loops", [1, 0])
def test_batch_knn_tc_ktruss(ctx, device_loops):
    """The batched workload's own graph family: uneven k-NN graphs, TC + 4-truss."""
    n, dim = _uneven_sizes(40, 32, 700, seed=21)
    U, voff = ga.gen_knn_batch(ctx, n, dim, k=30, seed=4)
    ctx.set_option(ga.OPT_DEVICE_LOOPS, device_loops)
    try:
        tcs = ga.batch_tc("msa", U, voff)
        C, iters = ga.batch_ktruss("msa", U, voff, 4)
    finally:
        ctx.set_option(ga.OPT_DEVICE_LOOPS, 1)
    rst, col, _ = U.download()
    blocks = ga.split_blocks(rst, col, voff)
    cr, cc, _ = C.download()
    got = ga.split_blocks(cr, cc, voff)
    solo = _solo_ktruss(ctx, "msa", blocks, 4)
    for g, (m, r, c) in enumerate(blocks):
        G = ga.Csr.upload(ctx, m, m, r, c, np.ones(len(c), np.int32))
        assert tcs[g] == ga.tc("dot", G, per_row=False)[0]
        assert iters[g] == solo[g][2]
        assert np.array_equal(got[g][1], solo[g][0]) and np.array_equal(got[g][2], solo[g][1])


def test_batch_rejects_bad_offsets(ctx):
    host, dev = _mixed_parts(ctx)
    U, voff = ga.block_diag(ctx, dev)
    bad = voff.copy()
    bad[-1] -= 1
    with pytest.raises(ga.GaError) as e:
        ga.batch_tc("msa", U, bad)
    assert e.value.code == ga.ERR_INVALID_ARG
    bad = voff.copy()
    bad[2], bad[3] = bad[3], bad[2]
    with pytest.raises(ga.GaError):
        ga.batch_ktruss("msa", U, bad, 4)


def test_knn_tiled_matches_cta(ctx):
    """The tiled generator kernel (graphs above 4,096 points) picks the same
    neighbours as the CTA-per-point kernel."""
    n, dim = _uneven_sizes(6, 2, 900, seed=8)
    U1, v1 = ga.gen_knn_batch(ctx, n, dim, k=30, seed=3)
    ctx.set_option(ga.OPT_KNN_TILED, 1)
    try:
        U2, v2 = ga.gen_knn_batch(ctx, n, dim, k=30, seed=3)
    finally:
        ctx.set_option(ga.OPT_KNN_TILED, 0)
    assert np.array_equal(v1, v2)
    assert all(np.array_equal(a, b) for a, b in zip(U1.download(), U2.download()))


def test_knn_large_graph(ctx):
    n = np.array([6000, 100], np.int32)
    U, voff = ga.gen_knn_batch(ctx, n, np.array([16, 5], np.int32), k=30, seed=11)
    rst, col, _ = U.download()
    for g, (m, r, c) in enumerate(ga.split_blocks(rst, col, voff)):
        assert m == n[g]
        _check_knn_structure(m, r, c, 30)


def test_batch_ktruss_per_graph_k(ctx):
    host, dev = _mixed_parts(ctx)
    U, voff = ga.block_diag(ctx, dev)
    ks = [3, 4, 5, 6, 7, 8, 4][:len(host)]
    C, iters = ga.batch_ktruss_k("msa", U, voff, ks)
    cr, cc, _ = C.download()
    got = ga.split_blocks(cr, cc, voff)
    for g, (G, k) in enumerate(zip(host, ks)):
        Cs, it = ga.ktruss("msa", dev[g], k)
        sr, sc, _ = Cs.download()
        assert iters[g] == it, g
        assert np.array_equal(got[g][1], sr) and np.array_equal(got[g][2], sc), g


def test_batch_bc_matches_single(ctx):
    host, dev = _mixed_parts(ctx)
    U, voff = ga.block_diag(ctx, dev)
    rng = np.random.default_rng(17)
    srcs = [rng.choice(G.m, min(G.m, 9), replace=False) for G in host]
    got = ga.batch_bc(U, voff, srcs)
    for g, (G, Gd, src) in enumerate(zip(host, dev, srcs)):
        ref = ga.bc(Gd, src)
        part = got[voff[g]:voff[g + 1]]
        assert np.all(np.abs(part - ref) <= 1e-9 * np.maximum(np.abs(ref), 1.0)), g
        orc = oracle.bc_batch(G, src)
        assert np.all(np.abs(part - orc) <= 1e-9 * np.maximum(np.abs(orc), 1.0)), g


def test_batch_bc_uneven_source_counts(ctx):
    """Graphs of a batch with different source counts share source columns:
    a graph with no sources (zero scores), one with 40 (a partly used second
    column word), one with 33, with 1 and with all its vertices; each part
    equals the graph alone and the FP64 oracle within 1e-9."""
    host, dev = _mixed_parts(ctx)
    rng = np.random.default_rng(23)
    counts = [40, 1, 33, 0, 5, 3, 120]
    srcs = [rng.choice(G.m, min(G.m, c), replace=False) for G, c in zip(host, counts)]
    U, voff = ga.block_diag(ctx, dev)
    got = ga.batch_bc(U, voff, srcs)
    for g, (G, Gd, src) in enumerate(zip(host, dev, srcs)):
        part = got[voff[g]:voff[g + 1]]
        if len(src) == 0:
            assert not np.any(part), g
            continue
        ref = ga.bc(Gd, src)
        assert np.all(np.abs(part - ref) <= 1e-9 * np.maximum(np.abs(ref), 1.0)), g
        orc = oracle.bc_batch(G, src)
        assert np.all(np.abs(part - orc) <= 1e-9 * np.maximum(np.abs(orc), 1.0)), g


def test_batch_bc_many_graphs(ctx):
    """More sources in all than one BC call takes (1,024): 48 k-NN graphs
    with 32 sources each, as the request server batches them."""
    n, dim = [int(x) for x in np.random.default_rng(5).integers(40, 400, 48)], [6] * 48
    U, voff = ga.gen_knn_batch(ctx, n, dim, k=30, seed=31)
    rst, col, _ = U.download()
    rng = np.random.default_rng(8)
    srcs = [rng.choice(m, 32, replace=False) for m in n]
    got = ga.batch_bc(U, voff, srcs)
    for g, (m, r, c) in enumerate(ga.split_blocks(rst, col, voff)):
        if g % 6:
            continue  # every sixth graph against the oracle
        G = oracle.Csr(m, m, r, c, np.ones(len(c), np.int32))
        orc = oracle.bc_batch(G, srcs[g].astype(np.int32))
        part = got[voff[g]:voff[g + 1]]
        assert np.all(np.abs(part - orc) <= 1e-9 * np.maximum(np.abs(orc), 1.0)), g


@pytest.mark.parametrize("device_loops", [1, 0])
def test_batch_ktruss_frontier_per_graph_k(ctx, device_loops):
    """The batched GA_TRI k-truss on the frontier path (one listing over the
    union, then only the pruned edges' triangles; every graph with its own
    k, iteration count and bound) against the batched form that lists every
    triangle each iteration and against each graph alone: edge sets and
    iteration counts equal, graphs without vertices or edges included."""
    host, dev = _mixed_parts(ctx)
    host.append(csr_from_arrays(*ga.gen_knn(500, 8, 30, seed=12)))
    dev.append(to_device(ctx, host[-1]))
    U, voff = ga.block_diag(ctx, dev)
    ks = [3, 5, 4, 8, 6, 3, 7, 9]
    ctx.set_option(ga.OPT_DEVICE_LOOPS, device_loops)
    try:
        out = []
        for frontier in (1, 0):
            ctx.set_option(ga.OPT_KT_FRONTIER, frontier)
            C, iters = ga.batch_ktruss_k("tri", U, voff, ks)
            cr, cc, _ = C.download()
            out.append((list(iters), ga.split_blocks(cr, cc, voff)))
            C.free()
        (it1, b1), (it0, b0) = out
        assert it1 == it0
        for g, ((m1, r1, c1), (m0, r0, c0)) in enumerate(zip(b1, b0)):
            assert np.array_equal(r1, r0) and np.array_equal(c1, c0), f"graph {g}"
        for g, (G, Gd) in enumerate(zip(host, dev)):
            C, it = ga.ktruss("tri", Gd, ks[g])
            r, c, _ = C.download()
            assert it1[g] == it, f"graph {g}"
            assert np.array_equal(b1[g][1], r) and np.array_equal(b1[g][2], c), f"graph {g}"
    finally:
        ctx.set_option(ga.OPT_KT_FRONTIER, 1)
        ctx.set_option(ga.OPT_DEVICE_LOOPS, 1)
