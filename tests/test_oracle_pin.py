"""Pins the CPU oracle (oracle/oracle.c) to the reference.

1. Against the committed golden fixtures (generated from the unmodified
   reference by tests/golden/make_golden.py) - runs everywhere.
2. Against the live reference library (oracle/_ref) on fresh seeded inputs -
   runs where the reference sources were available at build time.
3. Against the known answers on the reference's own Matrix-Market graphs,
   from the committed copies of those graphs as the reference's reader
   returns them (tests/golden/reference_graphs.npz) - runs everywhere; the
   copies are checked against the files where the reference tree is present.
"""
import json
import os

import numpy as np
import pytest

import oracle
from graphs import random_csr, random_graph

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")

REF_DIR = oracle.reference_dir()
REF_GRAPHS = os.path.join(REF_DIR, "graphs") if REF_DIR else None


@pytest.fixture(scope="module")
def gold():
    oracle.build()
    data = np.load(os.path.join(GOLD, "synthetic.npz"))
    with open(os.path.join(GOLD, "synthetic.json")) as f:
        meta = json.load(f)
    return data, meta


def _csr(data, key, m=None, n=None):
    rst = data[key + "_rst"]
    mm = len(rst) - 1
    return oracle.Csr(mm if m is None else m, mm if n is None else n, rst, data[key + "_col"], data[key + "_val"])


def test_golden_tc_and_rows(gold):
    data, meta = gold
    for name, info in meta["graphs"].items():
        G = _csr(data, f"{name}_A")
        total, rows = oracle.tc_sandia(G)
        assert total == info["triangles"], name
        assert np.array_equal(rows, data[f"{name}_tc_rows"]), name


def test_golden_ktruss(gold):
    data, meta = gold
    for name, info in meta["graphs"].items():
        G = _csr(data, f"{name}_A")
        for kt in info["ktruss"]:
            C, it = oracle.ktruss(G, kt["k"])
            R = _csr(data, f"{name}_k{kt['k']}")
            assert it == kt["iters"], (name, kt)
            assert np.array_equal(C.rst, R.rst) and np.array_equal(C.col, R.col), (name, kt)
            assert np.array_equal(C.val, R.val), (name, kt)


def test_golden_square_and_bc(gold):
    data, meta = gold
    for name, info in meta["graphs"].items():
        G = _csr(data, f"{name}_A")
        assert np.array_equal(oracle.mxm_masked(G, G, G), data[f"{name}_sq_val"]), name
        bc = oracle.bc_batch(G, data[f"{name}_bc_sources"])
        ref = data[f"{name}_bc_f64"]
        assert np.all(np.abs(bc - ref) <= 1e-12 * np.maximum(np.abs(ref), 1.0)), name
        # the shipped FP32 reference agrees to single precision
        b = info["bc_f32_batch"]
        bc32 = oracle.bc_batch(G, np.arange(b, dtype=np.int32))
        r32 = data[f"{name}_bc_f32_batch"].astype(np.float64)
        assert np.all(np.abs(bc32 - r32) <= 1e-4 * np.maximum(np.abs(bc32), 1.0)), name


def test_golden_mxm_variants_and_cmask(gold):
    data, meta = gold
    for key in meta["mxm"]:
        A, B, M = (_csr(data, f"{key}_{x}") for x in "ABM")
        got = oracle.mxm_masked(A, B, M)
        for algo in range(4):
            ref = data[f"{key}_algo{algo}_val"]
            if key.endswith("i32"):
                assert np.array_equal(got, ref), (key, algo)
            else:
                assert np.allclose(got, ref, rtol=1e-12, atol=1e-12), (key, algo)
        C = oracle.mxm_cmask(A, B, M)
        R = _csr(data, f"{key}_cmask")
        assert np.array_equal(C.rst, R.rst) and np.array_equal(C.col, R.col), key
        if key.endswith("i32"):
            assert np.array_equal(C.val, R.val), key
        else:
            assert np.allclose(C.val, R.val, rtol=1e-12, atol=1e-12), key


needs_ref = pytest.mark.skipif(not oracle.ref_available(), reason="reference library not built here")


@needs_ref
def test_live_reference_random_mxm_and_cmask():
    rng = np.random.default_rng(99)
    for trial in range(15):
        n = int(rng.integers(1, 60))
        for dt in (np.int32, np.float64):
            A = random_csr(n, n, rng.random() * 0.3, rng, dt)
            B = random_csr(n, n, rng.random() * 0.3, rng, dt)
            M = random_csr(n, n, rng.random() * 0.5, rng, dt)
            got = oracle.mxm_masked(A, B, M)
            for algo in range(4):
                R = oracle.ref_mxm(algo, A, B, M)
                assert np.array_equal(R.rst, M.rst) and np.array_equal(R.col, M.col)
                if dt == np.int32:
                    assert np.array_equal(R.val, got), algo
                else:
                    assert np.allclose(R.val, got, rtol=1e-12, atol=1e-12), algo
            C, R = oracle.mxm_cmask(A, B, M), oracle.ref_cmask(A, B, M)
            assert np.array_equal(C.rst, R.rst) and np.array_equal(C.col, R.col)


@needs_ref
def test_live_reference_graph_algorithms():
    rng = np.random.default_rng(100)
    for n, p in ((30, 0.3), (120, 0.08), (200, 0.05)):
        G = random_graph(n, p, rng)
        assert oracle.tc_sandia(G)[0] == oracle.ref_tc(G)[0]
        for k in (3, 4, 5):
            C, it = oracle.ktruss(G, k)
            R, rit = oracle.ref_ktruss(G, k)
            assert it == rit and np.array_equal(C.col, R.col) and np.array_equal(C.rst, R.rst)
        src = rng.choice(n, 10, replace=False).astype(np.int32)
        assert np.allclose(oracle.bc_batch(G, src), oracle.ref_bc_f64(G, src), rtol=1e-12, atol=1e-12)


def _ref_graph(z, name, what):
    rst = z[f"{name}_{what}_rst"]
    m = len(rst) - 1
    col = z[f"{name}_{what}_col"]
    val = z[f"{name}_raw_val"] if what == "raw" else np.ones(len(col), np.int32)
    n = int(z[f"{name}_raw_n"][0]) if what == "raw" else m
    return oracle.Csr(m, n, rst, col, val)


def test_reference_graph_known_answers():
    """Triangles and the whole k-truss sequence (edge counts and iteration
    counts) of the reference's four graphs, prepared as the CLI prepares
    them, against the answers the reference printed."""
    from oracle import formats as F
    with open(os.path.join(GOLD, "reference_graphs.json")) as f:
        known = json.load(f)
    z = np.load(os.path.join(GOLD, "reference_graphs.npz"))
    # the table of known answers measured on the reference (triangles, k-truss)
    assert known["G43"]["triangles"] == 1392 and known["yeast_30NN"]["triangles"] == 180175
    assert known["iris_dataset_30NN"]["triangles"] == 25972 and known["cage3"]["triangles"] == 3
    oracle.build()
    for name, info in known.items():
        G = _ref_graph(z, name, "cli")
        # the oracle's restatement of the CLI's preparation of the raw graph
        L = F.lower_symmetrised(F.adjacency(_ref_graph(z, name, "raw")))
        assert np.array_equal(L.rst, G.rst) and np.array_equal(L.col, G.col), name
        assert G.nnz == info["nnz"]
        assert oracle.tc_sandia(G)[0] == info["triangles"], name
        for k, nnz, iters in info["ktruss"]:
            C, it = oracle.ktruss(G, k)
            assert (C.nnz, it) == (nnz, iters), (name, k)


@pytest.mark.skipif(not (oracle.ref_available() and REF_GRAPHS and os.path.isdir(REF_GRAPHS)),
                    reason="reference graphs not present")
def test_reference_graph_fixtures_match_files():
    """The committed copies equal the reference's reading of its files."""
    z = np.load(os.path.join(GOLD, "reference_graphs.npz"))
    for name in ("G43", "cage3", "iris_dataset_30NN", "yeast_30NN"):
        path = os.path.join(REF_GRAPHS, name + ".mtx")
        R, code = oracle.ref_read_raw(path, "mtx")
        assert code == z[f"{name}_matcode"].tobytes()
        assert np.array_equal(R.rst, z[f"{name}_raw_rst"]) and np.array_equal(R.col, z[f"{name}_raw_col"])
        assert np.array_equal(R.val.view(np.int64), z[f"{name}_raw_val"].view(np.int64))
        C = oracle.ref_read_mtx(path)
        assert np.array_equal(C.rst, z[f"{name}_cli_rst"]) and np.array_equal(C.col, z[f"{name}_cli_col"])


def test_bc_all_sources_pins():
    """All-source BC (betweenness_centrality.h:5-123) by the oracle, FP64:
    equal to the sum of its batched runs over the blocks, to exact Brandes
    (networkx, counting ordered pairs on an undirected graph: twice its
    unnormalised score), and, where the reference was built, to the shipped
    FP32 reference within single precision."""
    oracle.build()
    rng = np.random.default_rng(41)
    G = random_graph(120, 0.05, rng)
    full = oracle.bc_all(G, 32)
    acc = np.zeros(G.m)
    for i in range(0, G.m, 32):
        acc += oracle.bc_batch(G, np.arange(i, min(G.m, i + 32), dtype=np.int32))
    assert np.allclose(full, acc, rtol=1e-12, atol=1e-12)
    assert np.allclose(oracle.bc_all(G, 7), full, rtol=1e-10, atol=1e-9)  # block size: rounding only
    nx = pytest.importorskip("networkx")
    H = nx.Graph()
    H.add_nodes_from(range(G.m))
    for i in range(G.m):
        for j in G.col[G.rst[i]:G.rst[i + 1]]:
            H.add_edge(i, int(j))
    exact = nx.betweenness_centrality(H, normalized=False)
    assert np.allclose(full, [2 * exact[v] for v in range(G.m)], rtol=1e-9, atol=1e-9)
    if oracle.ref_available():
        ref = oracle.ref_bc_all_f32(G, 32).astype(np.float64)
        assert np.allclose(full, ref, rtol=2e-5, atol=2e-3)
