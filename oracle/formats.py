"""CPU restatement of the reference's graph-file readers and writer (test
infrastructure only: the product never imports this module).

Follows include/matrix.h of UAlex322/GraphAlgo:
  * Matrix Market coordinate files, read_mtx_to_crs (matrix.h:280-417):
    banner and size line through mmio (src/mmio.cpp), then whitespace-
    separated entries "i j [v]" (1-based); self-loops are dropped
    (matrix.h:355-358, 373-376); a symmetric file stores each entry and its
    mirror, the mirror right after it (matrix.h:339-346, 379-386); rows keep
    that expanded order (a stable counting placement, matrix.h:396-408);
    pattern files get value 1. Complex and array files and non-square
    matrices are refused (matrix.h:301-309).
  * binary CSR, read_bin_to_crs / write_crs_to_bin (matrix.h:441-482,
    259-277): 4 matcode bytes, m, n, nz as 8-byte integers, Rst (m+1 int32),
    Col (nz int32), Val (nz values of the matrix's value type).
  * the CLI's value type (src/main.cpp:279-310): "real" files and binary files
    whose matcode[2] is 'R' hold doubles, everything else int32.
  * the CLI's preparation: build_adjacency_matrix (matrix.h:679-698, every
    value 1) and, for every action but BC, build_symm_from_lower(
    extract_lower_triangle(.)) (src/main.cpp:221-222).
"""
from __future__ import annotations

import struct

import numpy as np

from . import Csr


def _place(m: int, rows: np.ndarray, cols: np.ndarray, vals: np.ndarray, n: int) -> Csr:
    """Row-major CSR keeping, inside each row, the order of the input list."""
    order = np.argsort(rows, kind="stable")
    rst = np.zeros(m + 1, np.int32)
    np.cumsum(np.bincount(rows, minlength=m), out=rst[1:])
    return Csr(m, n, rst, cols[order].astype(np.int32), vals[order])


def mtx_banner(path: str):
    """(matcode bytes, m, n, nz, token list of the entries)."""
    with open(path, "rb") as f:
        data = f.read()
    lines = data.split(b"\n")
    head = lines[0].split()
    if len(head) != 5 or head[0].lower() != b"%%matrixmarket" or head[1].lower() != b"matrix":
        raise ValueError("not a Matrix Market file")
    fmt, field, sym = head[2].lower(), head[3].lower(), head[4].lower()
    code = b"M" + {b"coordinate": b"C", b"array": b"A"}[fmt] + \
        {b"real": b"R", b"integer": b"I", b"pattern": b"P", b"complex": b"C"}[field] + \
        {b"general": b"G", b"symmetric": b"S", b"skew-symmetric": b"K", b"hermitian": b"H"}[sym]
    k = 1
    while k < len(lines) and (lines[k].startswith(b"%") or not lines[k].strip()):
        k += 1
    m, n, nz = (int(t) for t in lines[k].split()[:3])
    body = b"\n".join(lines[k + 1:])
    return code, m, n, nz, body.split()


def read_mtx_raw(path: str) -> tuple[Csr, bytes]:
    """The matrix as read_mtx_to_crs builds it, values float64 for real files
    and int32 otherwise, with the file's matcode."""
    code, m, n, nz, tok = mtx_banner(path)
    if code[1:2] != b"C" or code[2:3] == b"C":
        raise ValueError("unsupported Matrix Market type")
    if m != n:
        raise ValueError("not a square matrix")
    per = 2 if code[2:3] == b"P" else 3
    if len(tok) < per * nz:
        raise ValueError("truncated entries")
    t = tok[: per * nz]
    i = np.array([int(x) for x in t[0::per]], np.int64) - 1
    j = np.array([int(x) for x in t[1::per]], np.int64) - 1
    real = code[2:3] == b"R"
    if per == 2:
        v = np.ones(nz, np.int32)
    elif real:
        v = np.array([float(x) for x in t[2::per]], np.float64)
    else:
        v = np.array([int(x) for x in t[2::per]], np.int32)
    keep = i != j
    i, j, v = i[keep], j[keep], v[keep]
    if code[3:4] == b"S":
        # entry, then its mirror
        i2 = np.empty(2 * len(i), np.int64)
        j2 = np.empty_like(i2)
        i2[0::2], i2[1::2] = i, j
        j2[0::2], j2[1::2] = j, i
        v = np.repeat(v, 2)
        i, j = i2, j2
    return _place(m, i, j, v, n), code


def read_bin_raw(path: str) -> tuple[Csr, bytes]:
    with open(path, "rb") as f:
        data = f.read()
    code = data[:4]
    m, n, nz = struct.unpack_from("<QQQ", data, 4)
    off = 28
    rst = np.frombuffer(data, np.int32, m + 1, off).copy()
    off += 4 * (m + 1)
    col = np.frombuffer(data, np.int32, nz, off).copy()
    off += 4 * nz
    dt = np.float64 if code[2:3] == b"R" else np.int32
    val = np.frombuffer(data, dt, nz, off).copy()
    return Csr(m, n, rst, col, val), code


def write_bin(path: str, A: Csr, code: bytes) -> None:
    with open(path, "wb") as f:
        f.write(code[:4])
        f.write(struct.pack("<QQQ", A.m, A.n, A.nnz))
        f.write(np.ascontiguousarray(A.rst, np.int32).tobytes())
        f.write(np.ascontiguousarray(A.col[: A.nnz], np.int32).tobytes())
        f.write(np.ascontiguousarray(A.val[: A.nnz]).tobytes())


def adjacency(A: Csr) -> Csr:
    return Csr(A.m, A.n, A.rst.copy(), A.col.copy(), np.ones(A.nnz, np.int32))


def lower_symmetrised(A: Csr) -> Csr:
    """build_symm_from_lower(extract_lower_triangle(A)) for rows sorted by
    column: the entries below the diagonal and their mirrors."""
    from . import extract_lower, symm_from_lower
    return symm_from_lower(extract_lower(A))


def sort_rows(A: Csr, merge_duplicates: bool = True) -> Csr:
    """Columns ascending within each row (stable); with `merge_duplicates`
    equal columns of a row collapse onto the first one's value."""
    rows = np.repeat(np.arange(A.m, dtype=np.int64), np.diff(A.rst.astype(np.int64)))
    col = A.col[: A.nnz].astype(np.int64)
    order = np.lexsort((col, rows))
    r, c, v = rows[order], col[order], A.val[: A.nnz][order]
    if merge_duplicates and len(r):
        first = np.ones(len(r), bool)
        first[1:] = (r[1:] != r[:-1]) | (c[1:] != c[:-1])
        r, c, v = r[first], c[first], v[first]
    rst = np.zeros(A.m + 1, np.int32)
    np.cumsum(np.bincount(r, minlength=A.m), out=rst[1:])
    return Csr(A.m, A.n, rst, c.astype(np.int32), v)


def from_edges(m: int, n: int, src, dst, val=None, mirror=False, drop_loops=False, lower_only=False) -> Csr:
    """Edge list to CSR with the product's ingestion rules: each edge (s, d)
    stands for (s, d) and, with `mirror`, (d, s); loops are dropped with
    `drop_loops` or `lower_only`; `lower_only` keeps the entries below the
    diagonal, each followed by its mirror (build_symm_from_lower(
    extract_lower_triangle(.))); rows are sorted and repeated entries merge
    onto the value of the earliest edge."""
    src = np.asarray(src, np.int64)
    dst = np.asarray(dst, np.int64)
    v = np.ones(len(src), np.int32) if val is None else np.asarray(val)
    eidx = np.arange(len(src))
    cand = [(src, dst)] + ([(dst, src)] if mirror else [])
    rows, cols, edge = [], [], []
    for a, b in cand:
        keep = np.ones(len(a), bool)
        if drop_loops or lower_only:
            keep &= a != b
        if lower_only:
            keep &= a > b
        rows.append(a[keep]); cols.append(b[keep]); edge.append(eidx[keep])
        if lower_only:
            rows.append(b[keep]); cols.append(a[keep]); edge.append(eidx[keep])
    r = np.concatenate(rows) if rows else np.zeros(0, np.int64)
    c = np.concatenate(cols) if cols else np.zeros(0, np.int64)
    e = np.concatenate(edge) if edge else np.zeros(0, np.int64)
    order = np.argsort(e, kind="stable")  # entries in edge order
    return sort_rows(_place(m, r[order], c[order], v[e[order]], n))
