"""The CUDA path on the reference's own four graphs (G43, cage3,
iris_dataset_30NN, yeast_30NN; SuiteSparse Matrix Collection matrices shipped
in the reference's graphs/ directory).

Inputs are the committed copies of each graph as the reference's reader
returns it (tests/golden/reference_graphs.npz, made by
tests/golden/make_golden.py). The CLI's preparation (build_adjacency_matrix,
then build_symm_from_lower(extract_lower_triangle(A)), src/main.cpp:221-222)
runs on the device, by the primitives and through a binary CSR file read
back with the preparation flags; both must give the reference's prepared
graph. Then triangle counts and the whole k-truss sequence (edge counts and
the iteration counts the reference prints) must equal the known answers in
tests/golden/reference_graphs.json, and the edge sets the oracle's.
"""
import json
import os

import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["G43", "cage3", "iris_dataset_30NN", "yeast_30NN"]

with open(os.path.join(GOLD, "reference_graphs.json")) as _f:
    KNOWN = json.load(_f)
Z = np.load(os.path.join(GOLD, "reference_graphs.npz"))


def _raw(name):
    rst = Z[f"{name}_raw_rst"]
    return len(rst) - 1, int(Z[f"{name}_raw_n"][0]), rst, Z[f"{name}_raw_col"], Z[f"{name}_raw_val"]


def _cli(name):
    rst = Z[f"{name}_cli_rst"]
    m = len(rst) - 1
    return oracle.Csr(m, m, rst, Z[f"{name}_cli_col"], np.ones(len(Z[f"{name}_cli_col"]), np.int32))


@pytest.fixture(scope="module")
def prepared(ctx):
    """Each graph prepared on the device by the primitives."""
    out = {}
    for name in NAMES:
        m, n, rst, col, val = _raw(name)
        R = ga.Csr.upload(ctx, m, n, rst, col, val)
        A = ga.adjacency(R)
        L = ga.extract_lower(A)
        out[name] = ga.symm_from_lower(L)
    return out


@pytest.mark.parametrize("name", NAMES)
def test_device_preparation(ctx, prepared, name, tmp_path):
    G = _cli(name)
    r, c, v = prepared[name].download()
    assert np.array_equal(r, G.rst) and np.array_equal(c, G.col) and np.all(v == 1)
    # the same through a binary CSR file read with the preparation flags
    m, n, rst, col, val = _raw(name)
    R = ga.Csr.upload(ctx, m, n, rst, col, val)
    path = str(tmp_path / (name + ".bin"))
    ga.write_bin(R, path, Z[f"{name}_matcode"].tobytes())
    B, code = ga.read_bin(ctx, path, ga.EDGES_LOWER_SYMM | ga.EDGES_UNIT)
    assert code == Z[f"{name}_matcode"].tobytes()
    r2, c2, _ = B.download()
    assert np.array_equal(r2, G.rst) and np.array_equal(c2, G.col)


@pytest.mark.parametrize("algo", ["tri", "dot", "msa", "mca", "heap", "hybrid"])
@pytest.mark.parametrize("name", NAMES)
def test_triangles(prepared, name, algo):
    total, rows = ga.tc(algo, prepared[name])
    assert total == KNOWN[name]["triangles"]
    ref_total, ref_rows = oracle.tc_sandia(_cli(name))
    assert total == ref_total and np.array_equal(rows, ref_rows)


@pytest.mark.parametrize("algo", ["tri", "msa"])
@pytest.mark.parametrize("name", NAMES)
def test_ktruss_sequence(prepared, name, algo):
    """Every k from 3 until the truss is empty, each from the prepared graph
    (the reference CLI's k-truss action): edge count and iteration count as
    the reference printed them, edge sets equal to the oracle's."""
    G = _cli(name)
    A = prepared[name]
    for k, nnz, iters in KNOWN[name]["ktruss"]:
        C, it = ga.ktruss(algo, A, k)
        assert (C.nnz, it) == (nnz, iters), (k, C.nnz, it)
        R, rit = oracle.ktruss(G, k)
        r, c, _ = C.download()
        assert rit == it and np.array_equal(r, R.rst) and np.array_equal(c, R.col), k
        C.free()
