"""Device ingestion: edge lists, Matrix Market and binary CSR files to CSR on
the GPU, against the reference's own reading of the committed fixtures
(tests/golden/formats) and the oracle's restatement of the rules. Indices and
integer values bit-exact; real values bit-exact (correctly rounded parsing)."""
import json
import os

import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle
from oracle import formats as F

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
FMT = os.path.join(GOLD, "formats")
with open(os.path.join(GOLD, "formats.json")) as _f:
    META = json.load(_f)
Z = np.load(os.path.join(GOLD, "formats.npz"))
NAMES = sorted(META)
SORTED = ("pat_sym", "real_sym")  # files whose rows the reference reads sorted


def golden(name, what):
    rst = Z[f"{name}_{what}_rst"]
    return oracle.Csr(len(rst) - 1, META[name]["m"], rst, Z[f"{name}_{what}_col"], Z[f"{name}_{what}_val"])


def assert_csr(D, E):
    """Device matrix D equals oracle matrix E (values compared bit for bit)."""
    rst, col, val = D.download()
    assert np.array_equal(rst, E.rst), "row starts"
    assert np.array_equal(col, E.col[: E.nnz]), "columns"
    ev = np.asarray(E.val[: E.nnz])
    if val.dtype == np.float64:
        assert np.array_equal(val.view(np.int64), ev.astype(np.float64).view(np.int64)), "values"
    else:
        assert np.array_equal(val, ev.astype(val.dtype)), "values"


@pytest.mark.parametrize("name", NAMES)
def test_read_mtx_matches_reference(ctx, name):
    A, code = ga.read_mtx(ctx, os.path.join(FMT, name + ".mtx"))
    assert code.decode() == META[name]["matcode"]
    R = golden(name, "raw")
    assert A.dtype == (ga.FP64 if code[2:3] == b"R" else ga.INT32)
    # the reference's matrix with rows sorted and repeated entries merged
    assert_csr(A, F.sort_rows(R))
    if name in SORTED:
        assert A.nnz == R.nnz


@pytest.mark.parametrize("name", NAMES)
def test_read_mtx_cli_preparation(ctx, name):
    A, _ = ga.read_mtx(ctx, os.path.join(FMT, name + ".mtx"), ga.EDGES_LOWER_SYMM | ga.EDGES_UNIT)
    U, _ = ga.read_mtx(ctx, os.path.join(FMT, name + ".mtx"), ga.EDGES_UNIT)
    assert A.dtype == ga.INT32 and U.dtype == ga.INT32
    S = F.sort_rows(golden(name, "raw"))
    assert_csr(A, F.lower_symmetrised(F.adjacency(S)))
    assert_csr(U, F.adjacency(S))
    if name in SORTED:
        assert_csr(A, golden(name, "cli1"))
        assert_csr(U, golden(name, "cli0"))


@pytest.mark.parametrize("name", NAMES)
def test_read_bin_matches_reference(ctx, name, tmp_path):
    path = os.path.join(FMT, name + ".bin")
    A, code = ga.read_bin(ctx, path)
    assert code.decode() == META[name]["bin_matcode"]
    assert_csr(A, F.sort_rows(golden(name, "bin")))
    L, _ = ga.read_bin(ctx, path, ga.EDGES_LOWER_SYMM | ga.EDGES_UNIT)
    assert_csr(L, F.lower_symmetrised(F.adjacency(F.sort_rows(golden(name, "bin")))))
    # a file whose rows are sorted and duplicate-free is written back byte for byte
    out = tmp_path / "w.bin"
    ga.write_bin(A, str(out), code)
    if name in SORTED:
        with open(path, "rb") as f:
            assert out.read_bytes() == f.read()
    B, _ = ga.read_bin(ctx, str(out))
    assert_csr(B, F.sort_rows(golden(name, "bin")))


def test_tc_on_read_graph(ctx):
    A, _ = ga.read_mtx(ctx, os.path.join(FMT, "pat_sym.mtx"), ga.EDGES_LOWER_SYMM | ga.EDGES_UNIT)
    total, rows = ga.tc("msa", A)
    G = golden("pat_sym", "cli1")
    ref_total, ref_rows = oracle.tc_sandia(G)
    assert total == ref_total and np.array_equal(rows, ref_rows)


def _random_edges(rng, m, n, ne, hub=None, hub_deg=0):
    src = rng.integers(0, m, ne).astype(np.int32)
    dst = rng.integers(0, n, ne).astype(np.int32)
    if hub is not None:
        src = np.concatenate([src, np.full(hub_deg, hub, np.int32)])
        dst = np.concatenate([dst, rng.integers(0, n, hub_deg).astype(np.int32)])
    dup = rng.choice(len(src), len(src) // 10, replace=False)
    src = np.concatenate([src, src[dup]])
    dst = np.concatenate([dst, dst[dup]])
    order = rng.permutation(len(src))
    return src[order], dst[order]


@pytest.mark.parametrize("flags", [0, ga.EDGES_DROP_LOOPS, ga.EDGES_MIRROR, ga.EDGES_MIRROR | ga.EDGES_DROP_LOOPS,
                                   ga.EDGES_LOWER_SYMM, ga.EDGES_LOWER_SYMM | ga.EDGES_MIRROR,
                                   ga.EDGES_UNIT | ga.EDGES_MIRROR])
@pytest.mark.parametrize("dtype", [np.int32, np.float64])
def test_from_edges_rules(ctx, flags, dtype):
    rng = np.random.default_rng(flags * 7 + (dtype == np.float64))
    m = 700
    src, dst = _random_edges(rng, m, m, 6000, hub=5, hub_deg=20000)
    val = (rng.integers(-9, 9, len(src)) if dtype == np.int32 else rng.standard_normal(len(src))).astype(dtype)
    A = ga.csr_from_edges(ctx, m, m, src, dst, val, flags)
    E = F.from_edges(m, m, src, dst, None if flags & ga.EDGES_UNIT else val,
                     mirror=bool(flags & ga.EDGES_MIRROR), drop_loops=bool(flags & ga.EDGES_DROP_LOOPS),
                     lower_only=bool(flags & ga.EDGES_LOWER_SYMM))
    assert A.dtype == (ga.INT32 if flags & ga.EDGES_UNIT else ga._DT[np.dtype(dtype)])
    assert_csr(A, E)


def test_from_edges_rectangular_and_empty(ctx):
    rng = np.random.default_rng(3)
    src, dst = _random_edges(rng, 50, 3000, 4000, hub=7, hub_deg=40000)
    A = ga.csr_from_edges(ctx, 50, 3000, src, dst)
    assert_csr(A, F.from_edges(50, 3000, src, dst))
    E = ga.csr_from_edges(ctx, 10, 10, np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert E.nnz == 0 and np.array_equal(E.download()[0], np.zeros(11, np.int32))
    Z0 = ga.csr_from_edges(ctx, 0, 0, np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert Z0.nnz == 0


def test_from_edges_errors(ctx):
    with pytest.raises(ga.GaError) as e:
        ga.csr_from_edges(ctx, 4, 4, [0, 4], [1, 1])
    assert e.value.code == ga.ERR_INVALID_ARG
    with pytest.raises(ga.GaError) as e:
        ga.csr_from_edges(ctx, 4, 5, [0], [1], flags=ga.EDGES_MIRROR)
    assert e.value.code == ga.ERR_SHAPE
    with pytest.raises(ga.GaError) as e:
        ga.csr_from_edges(ctx, 4, 4, [0], [1], flags=64)
    assert e.value.code == ga.ERR_INVALID_ARG


def _write_mtx(path, header, size, lines, end="\n"):
    with open(path, "w", newline="") as f:
        f.write(end.join([header, size] + lines) + end)


def test_malformed_mtx_files(ctx, tmp_path):
    p = str(tmp_path / "bad.mtx")
    cases = [
        ("%%MatrixMarket matrix coordinate pattern general", "3 3 3", ["1 2", "2 3"], ga.ERR_INVALID_ARG),
        ("%%MatrixMarket matrix coordinate pattern general", "3 3 2", ["1 2", "2 4"], ga.ERR_INVALID_ARG),
        ("%%MatrixMarket matrix coordinate pattern general", "3 3 2", ["1 2", "x 3"], ga.ERR_INVALID_ARG),
        ("%%MatrixMarket matrix coordinate integer general", "3 3 1", ["1 2 9999999999"], ga.ERR_INVALID_ARG),
        ("%%MatrixMarket matrix coordinate real general", "3 3 1", ["1 2 1.5x"], ga.ERR_INVALID_ARG),
        ("%%MatrixMarket matrix coordinate complex general", "3 3 1", ["1 2 1 0"], ga.ERR_UNSUPPORTED),
        ("%%MatrixMarket matrix array real general", "3 3", ["1"], ga.ERR_UNSUPPORTED),
        ("%%MatrixMarket matrix coordinate pattern general", "3 4 1", ["1 2"], ga.ERR_SHAPE),
        ("%%NotMatrixMarket matrix coordinate pattern general", "3 3 1", ["1 2"], ga.ERR_INVALID_ARG),
    ]
    for header, size, lines, code in cases:
        _write_mtx(p, header, size, lines)
        with pytest.raises(ga.GaError) as e:
            ga.read_mtx(ctx, p)
        assert e.value.code == code, (header, size, lines)
    with pytest.raises(ga.GaError):
        ga.read_mtx(ctx, str(tmp_path / "missing.mtx"))


def test_mtx_layout_variants(ctx, tmp_path):
    """Blank lines, CRLF, tabs, several entries on one line and no final
    newline: the body is whitespace-separated tokens."""
    p = str(tmp_path / "v.mtx")
    with open(p, "w", newline="") as f:
        f.write("%%MatrixMarket matrix coordinate real general\r\n%c\r\n\r\n4 4 5\r\n"
                "1 2 0.5\r\n\r\n2\t3 -1e-3  3 1 .25 4 4 7\n2 1 1e-40")
    A, code = ga.read_mtx(ctx, p)
    assert code == b"MCRG"
    E = F.from_edges(4, 4, [0, 1, 2, 3, 1], [1, 2, 0, 3, 0], np.array([0.5, -1e-3, 0.25, 7.0, 1e-40]),
                     drop_loops=True)
    assert_csr(A, E)


@pytest.mark.parametrize("field", ["pattern", "integer", "real"])
def test_large_generated_mtx(ctx, tmp_path, field):
    """A 2^17-vertex R-MAT edge list with hubs written as Matrix Market
    text: the device reader equals the restatement of the rules."""
    m, rst, col = ga.gen_rmat(17, 8, seed=11)
    rows = np.repeat(np.arange(m, dtype=np.int64), np.diff(rst))
    keep = rows > col  # lower triangle, written as a symmetric file
    i, j = rows[keep] + 1, col[keep].astype(np.int64) + 1
    rng = np.random.default_rng(5)
    order = rng.permutation(len(i))
    i, j = i[order], j[order]
    if field == "pattern":
        body = "\n".join(f"{a} {b}" for a, b in zip(i.tolist(), j.tolist()))
        vals = None
    elif field == "integer":
        vals = rng.integers(-100000, 100000, len(i)).astype(np.int32)
        body = "\n".join(f"{a} {b} {v}" for a, b, v in zip(i.tolist(), j.tolist(), vals.tolist()))
    else:
        vals = rng.standard_normal(len(i)) * 10.0 ** rng.integers(-8, 8, len(i))
        body = "\n".join(f"{a} {b} {v!r}" for a, b, v in zip(i.tolist(), j.tolist(), vals.tolist()))
        vals = np.array([float(repr(v)) for v in vals.tolist()])
    p = str(tmp_path / "big.mtx")
    with open(p, "w") as f:
        f.write(f"%%MatrixMarket matrix coordinate {field} symmetric\n{m} {m} {len(i)}\n{body}\n")
    A, _ = ga.read_mtx(ctx, p)
    E = F.from_edges(m, m, i - 1, j - 1, vals, mirror=True, drop_loops=True)
    assert_csr(A, E)
    assert A.nnz == 2 * len(i)


def test_transpose_with_long_columns(ctx):
    """Transposition sorts each output row; a column with 40,000 entries
    takes the long-row merge path."""
    rng = np.random.default_rng(8)
    m, n = 60000, 300
    src = np.arange(m, dtype=np.int32)
    dst = np.where(rng.random(m) < 0.67, 17, rng.integers(0, n, m)).astype(np.int32)
    val = rng.standard_normal(m)
    A = ga.csr_from_edges(ctx, m, n, src, dst, val)
    T = ga.transpose(A)
    E = oracle.transpose(F.from_edges(m, n, src, dst, val))
    assert_csr(T, E)


@pytest.mark.parametrize("scale,ef,seed", [(6, 4, 3), (12, 16, 7), (17, 16, 11)])
def test_rmat_device_equals_host(ctx, scale, ef, seed):
    """The device R-MAT builder gives the host generator's graph bit for bit
    (same random streams; chunks of 2^16 edges cross thread boundaries at
    scale 17)."""
    m, rst, col = ga.gen_rmat(scale, ef, seed=seed)
    A = ga.gen_rmat_device(ctx, scale, ef, seed=seed)
    assert A.shape == (m, m) and A.dtype == ga.INT32
    dr, dc, dv = A.download()
    assert np.array_equal(dr, rst) and np.array_equal(dc, col)
    assert np.all(dv == 1)


def test_rmat_device_errors(ctx):
    with pytest.raises(ga.GaError):
        ga.gen_rmat_device(ctx, 0, 16)
    with pytest.raises(ga.GaError):
        ga.gen_rmat_device(ctx, 10, 16, a=0.6, b=0.3, c=0.3)
