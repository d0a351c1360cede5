"""CPU checks of the graph-file formats: the oracle's restatement of the
reference's Matrix Market reader, binary reader and writer against what the
reference itself produced for the committed fixtures (tests/golden/formats),
and the ingestion entry points' argument checks (no GPU needed)."""
import json
import os

import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle
from oracle import formats as F

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
FMT = os.path.join(GOLD, "formats")
REF_DIR = oracle.reference_dir()
REF_GRAPHS = os.path.join(REF_DIR, "graphs") if REF_DIR else None

with open(os.path.join(GOLD, "formats.json")) as _f:
    META = json.load(_f)
Z = np.load(os.path.join(GOLD, "formats.npz"))


def golden(name, what):
    rst = Z[f"{name}_{what}_rst"]
    return oracle.Csr(len(rst) - 1, META[name]["m"], rst, Z[f"{name}_{what}_col"], Z[f"{name}_{what}_val"])


def same_bits(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.int64), b.view(np.int64))


@pytest.mark.parametrize("name", sorted(META))
def test_mtx_restatement_matches_reference(name):
    O, code = F.read_mtx_raw(os.path.join(FMT, name + ".mtx"))
    R = golden(name, "raw")
    assert code.decode() == META[name]["matcode"]
    assert np.array_equal(O.rst, R.rst) and np.array_equal(O.col, R.col)
    assert same_bits(O.val, R.val)


@pytest.mark.parametrize("name", sorted(META))
def test_bin_restatement_matches_reference(name, tmp_path):
    path = os.path.join(FMT, name + ".bin")
    B, code = F.read_bin_raw(path)
    R = golden(name, "bin")
    assert code.decode() == META[name]["bin_matcode"]
    assert np.array_equal(B.rst, R.rst) and np.array_equal(B.col, R.col) and same_bits(B.val, R.val)
    # the writer reproduces the reference's tobinary bytes from the raw read
    O, mcode = F.read_mtx_raw(os.path.join(FMT, name + ".mtx"))
    out = tmp_path / "x.bin"
    F.write_bin(str(out), O, mcode)
    with open(path, "rb") as f:
        assert out.read_bytes() == f.read()


@pytest.mark.parametrize("name", sorted(META))
def test_cli_preparation_on_sorted_rows(name):
    """The reference's CLI preparation equals the oracle's on files whose
    rows come out sorted (column-major files); on shuffled files the
    reference's extract_lower_triangle reads only the prefix of each row
    below the diagonal, so the product (which sorts first) follows the
    restatement on sorted rows instead."""
    O, _ = F.read_mtx_raw(os.path.join(FMT, name + ".mtx"))
    S = F.sort_rows(O, merge_duplicates=False)
    rows_sorted = np.array_equal(S.col, O.col)
    A = F.adjacency(S)
    R0 = golden(name, "cli0")
    if rows_sorted:
        assert np.array_equal(R0.col, A.col) and np.array_equal(R0.rst, A.rst)
        R1 = golden(name, "cli1")
        L = F.lower_symmetrised(A)
        assert np.array_equal(R1.rst, L.rst) and np.array_equal(R1.col, L.col)
    else:
        assert name in ("real_gen", "int_gen_dup", "int_sym_shuffled")


@pytest.mark.skipif(not (oracle.ref_available() and REF_GRAPHS and os.path.isdir(REF_GRAPHS)),
                    reason="reference graphs not present")
@pytest.mark.parametrize("g", ["G43", "cage3", "iris_dataset_30NN", "yeast_30NN"])
def test_mtx_restatement_on_reference_graphs(g):
    path = os.path.join(REF_GRAPHS, g + ".mtx")
    R, code = oracle.ref_read_raw(path, "mtx")
    O, ocode = F.read_mtx_raw(path)
    assert code == ocode
    assert np.array_equal(O.rst, R.rst) and np.array_equal(O.col, R.col) and same_bits(O.val, R.val)
    C = oracle.ref_read_cli(path, "mtx", True)
    L = F.lower_symmetrised(F.adjacency(O))
    assert np.array_equal(C.rst, L.rst) and np.array_equal(C.col, L.col)


def test_from_edges_rules():
    # (0,1) twice, a loop, an upper entry; lower-symmetrised keeps (1,0) and (2,1)
    src = [0, 1, 0, 2, 2, 1]
    dst = [1, 0, 1, 2, 1, 2]
    val = np.array([5, 6, 7, 8, 9, 10], np.int32)
    A = F.from_edges(3, 3, src, dst, val)
    assert A.rst.tolist() == [0, 1, 3, 5]
    assert A.col.tolist() == [1, 0, 2, 1, 2] and A.val.tolist() == [5, 6, 10, 9, 8]
    L = F.from_edges(3, 3, src, dst, val, lower_only=True)
    assert L.col.tolist() == [1, 0, 2, 1] and L.val.tolist() == [6, 6, 9, 9]
    M = F.from_edges(3, 3, src, dst, val, mirror=True, drop_loops=True)
    # (0,1) from edge 0 first, its mirror (1,0) from edge 0 before edge 1's
    assert M.col.tolist() == [1, 0, 2, 1] and M.val.tolist() == [5, 5, 9, 9]


def test_ingest_entry_points_reject_bad_arguments(built):
    L = ga.lib()
    import ctypes
    h = ctypes.c_void_p()
    assert L.ga_read_mtx(None, b"x.mtx", 0, None, ctypes.byref(h)) == ga.ERR_INVALID_ARG
    assert L.ga_read_bin(None, b"x.bin", 0, None, ctypes.byref(h)) == ga.ERR_INVALID_ARG
    assert L.ga_write_bin(None, None, None, b"x.bin") == ga.ERR_INVALID_ARG
    assert L.ga_csr_from_edges(None, ctypes.c_int64(1), ctypes.c_int64(1), ctypes.c_int64(0), None, None, None,
                               0, 0, ctypes.byref(h)) == ga.ERR_INVALID_ARG
    assert L.ga_csr_from_device_edges(None, ctypes.c_int64(1), ctypes.c_int64(1), ctypes.c_int64(1), None, None,
                                      None, 0, 0, ctypes.byref(h)) == ga.ERR_INVALID_ARG


@pytest.mark.parametrize("name", sorted(META))
def test_c_port_of_cli_reading_matches_reference(built, name):
    """oracle.read_mtx_cli (the CPU baseline of the ingestion benchmark)
    reproduces the reference CLI's reading, rows in the reference's order."""
    for sym in (0, 1):
        A = oracle.read_mtx_cli(os.path.join(FMT, name + ".mtx"), bool(sym))
        R = golden(name, f"cli{sym}")
        assert np.array_equal(A.rst, R.rst) and np.array_equal(A.col, R.col)
