#!/usr/bin/env python3
"""Regenerates the golden fixtures in this directory from the UNMODIFIED
reference (UAlex322/GraphAlgo), compiled from its own sources into
oracle/_ref/libref.so by oracle/build_ref.sh.

Inputs are seeded synthetic graphs made here with numpy (independent of the
product's generators). Outputs come from the reference's own functions:
  mxmm_msa / mxmm_mca / mxmm_heap (C.Val zero-filled first) / mxmm_naive,
  mxmm_msa_cmask, triangle_counting_masked_sandia and the row sums of its
  C<L> = L*L, k_truss (edge sets and printed iteration counts), and the
  batched BC both as shipped (FP32, sources 0..b-1) and with the reference's
  templates instantiated at double for an explicit source list.
For the four Matrix-Market graphs shipped with the reference (matrices of
the SuiteSparse Matrix Collection): the known answers (triangles, k-truss
edge counts and iterations, reference_graphs.json) and, as test inputs, each
graph as the reference's own reader returns it (row starts, columns, values
and type code) and after the CLI's preparation (reference_graphs.npz).
File formats: seeded Matrix Market files written here (formats/*.mtx), the
reference's raw reading and CLI preparation of each (formats.npz) and the
binary files its "tobinary" action writes for them (formats/*.bin).
Element-wise: the reference's eWiseAdd and VxM on seeded operands (ewise.npz).

    python tests/golden/make_golden.py            # everything
    python tests/golden/make_golden.py formats    # the file-format fixtures only
    python tests/golden/make_golden.py ewise      # eWiseAdd / VxM fixtures only
    python tests/golden/make_golden.py graphs     # the reference's four graphs only
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

REF_GRAPHS = os.path.join(os.environ.get("REF", "/root/reference"), "graphs")


def csr_from_dense(D, V=None, dtype=np.int32):
    m, n = D.shape
    rst = np.zeros(m + 1, np.int32)
    rst[1:] = np.cumsum((D != 0).sum(1))
    r, c = np.nonzero(D)
    val = (V[r, c] if V is not None else np.ones(len(c))).astype(dtype)
    return oracle.Csr(m, n, rst, c.astype(np.int32), val)


def sym_graph(n, p, rng):
    U = np.triu(rng.random((n, n)) < p, 1)
    return csr_from_dense(U | U.T)


def rmat_graph(scale, ef, rng, a=0.57, b=0.19, c=0.19):
    n = 1 << scale
    e = n * ef
    u = np.zeros(e, np.int64)
    v = np.zeros(e, np.int64)
    for _ in range(scale):
        r = rng.random(e)
        bu = (r >= a + b).astype(np.int64)
        bv = (((r >= a) & (r < a + b)) | (r >= a + b + c)).astype(np.int64)
        u = (u << 1) | bu
        v = (v << 1) | bv
    keep = u != v
    D = np.zeros((n, n), bool)
    D[u[keep], v[keep]] = True
    D = D | D.T
    return csr_from_dense(D)


def knn_graph(n, dim, k, rng):
    X = rng.standard_normal((n, dim))
    d2 = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d2, np.inf)
    nb = np.argsort(d2, axis=1, kind="stable")[:, :k]
    D = np.zeros((n, n), bool)
    D[np.repeat(np.arange(n), k), nb.ravel()] = True
    return csr_from_dense(D | D.T)


def pack(prefix, C, out):
    out[prefix + "_rst"] = C.rst
    out[prefix + "_col"] = C.col
    out[prefix + "_val"] = C.val


FORMATS = os.path.join(HERE, "formats")


def _fmt_real(x: float, style: int) -> str:
    """Real values in the spellings Matrix Market writers use, including the
    leading-dot form of the reference's own kNN graphs."""
    if style == 0:
        return repr(float(x))
    if style == 1:
        t = "%.16f" % x
        return t.replace("0.", ".", 1) if t.startswith("0.") else t.replace("-0.", "-.", 1)
    if style == 2:
        return "%.6e" % x
    if style == 3:
        return "%.17g" % x
    return "%.24f" % x  # more significant digits than the device's fast path takes


def write_formats(rng) -> dict:
    """Seeded Matrix Market files (this script's own content) and what the
    reference makes of them: its raw reader, its CLI preparation with and
    without the lower-triangle symmetrisation, and its tobinary output."""
    os.makedirs(FORMATS, exist_ok=True)
    files = {}

    def lower_pairs(n, p):
        U = np.tril(rng.random((n, n)) < p, -1)
        j, i = np.nonzero(U.T)  # column-major order: by column, then row
        return i + 1, j + 1

    # pattern symmetric, column-major lower triangle with a few diagonal
    # entries and comment lines (no blank line before the size line: the
    # reference's second pass, matrix.h:330-332, would take it for the size
    # line and read every entry one token off)
    i, j = lower_pairs(120, 0.06)
    diag = rng.choice(120, 5, replace=False) + 1
    lines = ["%%MatrixMarket matrix coordinate pattern symmetric", "% seeded test graph", "%"]
    body = [f"{a} {b}" for a, b in zip(i, j)] + [f"{d} {d}" for d in diag]
    lines.append(f"120 120 {len(body)}")
    files["pat_sym"] = "\n".join(lines + body) + "\n"

    # real symmetric in column-major order, values in mixed spellings
    i, j = lower_pairs(150, 0.08)
    v = rng.random(len(i)) * 0.2
    body = [f"{a} {b} {_fmt_real(x, k % 4)}" for k, (a, b, x) in enumerate(zip(i, j, v))]
    files["real_sym"] = "\n".join(["%%MatrixMarket matrix coordinate real symmetric",
                                   f"150 150 {len(body)}"] + body) + "\n"

    # real general, entries in random order (rows unsorted), CRLF line ends,
    # tabs, long and exponent-heavy values that leave the fast path
    n = 90
    D = rng.random((n, n)) < 0.07
    r, c = np.nonzero(D)
    order = rng.permutation(len(r))
    r, c = r[order] + 1, c[order] + 1
    vals = rng.standard_normal(len(r)) * 10.0 ** rng.integers(-30, 30, len(r))
    specials = ["-0", "2", "1E+2", "-1.5e-3", "3.0000000000000004", "1e-30", "0.000123456789012345678901",
                "+.5", "7.", "123456789012345678901234"]
    body = []
    for k, (a, b, x) in enumerate(zip(r, c, vals)):
        t = specials[k] if k < len(specials) else _fmt_real(x, k % 5)
        sep = "\t" if k % 7 == 0 else " "
        body.append(f"{a}{sep}{b} {t}")
    files["real_gen"] = "\r\n".join(["%%MatrixMarket matrix coordinate real general", f"{n} {n} {len(body)}"]
                                     + body) + "\r\n"

    # integer general with repeated (i, j) entries and negative values
    n = 60
    D = rng.random((n, n)) < 0.1
    r, c = np.nonzero(D)
    dup = rng.choice(len(r), 15, replace=False)
    r = np.concatenate([r, r[dup]]) + 1
    c = np.concatenate([c, c[dup]]) + 1
    iv = rng.integers(-1000, 1000, len(r))
    body = [f"{a} {b} {x}" for a, b, x in zip(r, c, iv)]
    files["int_gen_dup"] = "\n".join(["%%MatrixMarket matrix coordinate integer general",
                                      f"{n} {n} {len(body)}"] + body) + "\n"

    # integer symmetric with entries in random order
    i, j = lower_pairs(80, 0.1)
    order = rng.permutation(len(i))
    i, j = i[order], j[order]
    iv = rng.integers(1, 50, len(i))
    body = [f"{a} {b} {x}" for a, b, x in zip(i, j, iv)]
    files["int_sym_shuffled"] = "\n".join(["%%MatrixMarket matrix coordinate integer symmetric",
                                           f"80 80 {len(body)}"] + body) + "\n"

    out = {}
    meta = {}
    for name, text in files.items():
        path = os.path.join(FORMATS, name + ".mtx")
        with open(path, "w", newline="") as f:
            f.write(text)
        R, code = oracle.ref_read_raw(path, "mtx")
        pack(f"{name}_raw", R, out)
        for sym in (0, 1):
            pack(f"{name}_cli{sym}", oracle.ref_read_cli(path, "mtx", bool(sym)), out)
        binp = os.path.join(FORMATS, name + ".bin")
        oracle.ref_tobinary(path, "mtx", binp)
        B, bcode = oracle.ref_read_raw(binp, "bin")
        pack(f"{name}_bin", B, out)
        meta[name] = {"matcode": code.decode(), "bin_matcode": bcode.decode(), "m": R.m, "nnz": int(R.nnz)}
    np.savez_compressed(os.path.join(HERE, "formats.npz"), **out)
    with open(os.path.join(HERE, "formats.json"), "w") as f:
        json.dump(meta, f, indent=1)
    return meta


def write_ewise(rng) -> list:
    """The reference's eWiseAdd (unmasked; masked on operands that share a
    pattern, where its B-indexing slip is invisible) and VxM on seeded
    operands."""
    out = {}
    keys = []
    for t in range(3):
        m, n = int(rng.integers(20, 60)), int(rng.integers(20, 60))
        for dt, tag in ((np.int32, "i32"), (np.float64, "f64")):
            def mat(dens):
                D = rng.random((m, n)) < dens
                V = rng.integers(-3, 4, (m, n)) if dt == np.int32 else rng.standard_normal((m, n))
                return csr_from_dense(D, V, dt)
            A, B, M = mat(0.2), mat(0.2), mat(0.3)
            B2 = oracle.Csr(A.m, A.n, A.rst, A.col,
                            (rng.integers(-3, 4, A.nnz) if dt == np.int32 else rng.standard_normal(A.nnz)).astype(dt))
            key = f"ew{t}_{tag}"
            for nm, X in (("A", A), ("B", B), ("M", M), ("B2", B2)):
                pack(f"{key}_{nm}", X, out)
            pack(f"{key}_add", oracle.ref_ewise_add(A, B), out)
            pack(f"{key}_madd", oracle.ref_ewise_add(A, B2, M), out)
            x = (rng.integers(-5, 5, m) if dt == np.int32 else rng.standard_normal(m)).astype(dt)
            y = (rng.integers(-5, 5, n) if dt == np.int32 else rng.standard_normal(n)).astype(dt)
            out[f"{key}_x"], out[f"{key}_y"] = x, y
            out[f"{key}_vxm"] = oracle.ref_vxm(A, x, y)
            keys.append(key)
    np.savez_compressed(os.path.join(HERE, "ewise.npz"), **out)
    return keys


def write_reference_graphs() -> list:
    """Each reference graph as the reference reads it (read_mtx_to_crs,
    include/matrix.h:280-417: self-loops dropped, symmetric files mirrored;
    float64 values) and after the CLI's preparation (build_adjacency_matrix,
    then build_symm_from_lower(extract_lower_triangle(A)),
    src/main.cpp:221-222)."""
    out = {}
    names = []
    for g in sorted(os.listdir(REF_GRAPHS)):
        if not g.endswith(".mtx"):
            continue
        name = g[:-4]
        path = os.path.join(REF_GRAPHS, g)
        R, code = oracle.ref_read_raw(path, "mtx")
        out[f"{name}_raw_rst"] = R.rst
        out[f"{name}_raw_col"] = R.col
        out[f"{name}_raw_val"] = R.val
        out[f"{name}_raw_n"] = np.array([R.n], np.int64)
        out[f"{name}_matcode"] = np.frombuffer(code, np.uint8)
        C = oracle.ref_read_cli(path, "mtx", True)
        out[f"{name}_cli_rst"] = C.rst
        out[f"{name}_cli_col"] = C.col
        names.append(name)
    np.savez_compressed(os.path.join(HERE, "reference_graphs.npz"), **out)
    return names


def main():
    if oracle.build_ref() is None:
        raise SystemExit("reference sources not available; cannot regenerate fixtures")
    rng = np.random.default_rng(20261203)
    graphs = {
        "er300": sym_graph(300, 0.05, rng),
        "rmat9": rmat_graph(9, 8, rng),
        "knn200": knn_graph(200, 5, 12, rng),
        "dense40": sym_graph(40, 0.6, rng),
    }
    out = {}
    meta = {"graphs": {}, "mxm": []}
    for name, G in graphs.items():
        pack(f"{name}_A", G, out)
        total, rows = oracle.ref_tc(G)
        out[f"{name}_tc_rows"] = rows
        kt = []
        k = 3
        while True:
            R, it = oracle.ref_ktruss(G, k)
            pack(f"{name}_k{k}", R, out)
            kt.append({"k": k, "nnz": int(R.nnz), "iters": it})
            if R.nnz == 0:
                break
            k += 1
        sources = rng.choice(G.m, min(24, G.m), replace=False).astype(np.int32)
        out[f"{name}_bc_sources"] = sources
        out[f"{name}_bc_f64"] = oracle.ref_bc_f64(G, sources)
        b = min(16, G.m)
        out[f"{name}_bc_f32_batch"] = oracle.ref_bc_f32(G, b)
        sq = oracle.ref_mxm(0, G, G, G)
        out[f"{name}_sq_val"] = sq.val
        meta["graphs"][name] = {"m": G.m, "nnz": int(G.nnz), "triangles": total, "ktruss": kt,
                                "bc_f32_batch": b}
    # random square matrices with int and double values for the four variants
    for t in range(4):
        n = int(rng.integers(20, 70))
        for dt, tag in ((np.int32, "i32"), (np.float64, "f64")):
            mats = []
            for dens in (0.15, 0.15, 0.4):
                D = rng.random((n, n)) < dens
                V = rng.integers(-3, 4, (n, n)) if dt == np.int32 else rng.standard_normal((n, n))
                mats.append(csr_from_dense(D, V, dt))
            A, B, M = mats
            key = f"mxm{t}_{tag}"
            for nm, X in zip("ABM", mats):
                pack(f"{key}_{nm}", X, out)
            for algo in range(4):
                out[f"{key}_algo{algo}_val"] = oracle.ref_mxm(algo, A, B, M).val
            pack(f"{key}_cmask", oracle.ref_cmask(A, B, M), out)
            meta["mxm"].append(key)
    np.savez_compressed(os.path.join(HERE, "synthetic.npz"), **out)
    with open(os.path.join(HERE, "synthetic.json"), "w") as f:
        json.dump(meta, f, indent=1)
    # known answers on the reference's own graphs
    known = {}
    if os.path.isdir(REF_GRAPHS):
        for g in sorted(os.listdir(REF_GRAPHS)):
            if not g.endswith(".mtx"):
                continue
            G = oracle.ref_read_mtx(os.path.join(REF_GRAPHS, g))
            total, _ = oracle.ref_tc(G)
            kt = []
            k = 3
            while True:
                R, it = oracle.ref_ktruss(G, k)
                kt.append([k, int(R.nnz), it])
                if R.nnz == 0:
                    break
                k += 1
            known[g[:-4]] = {"m": G.m, "nnz": int(G.nnz), "triangles": total, "ktruss": kt}
        with open(os.path.join(HERE, "reference_graphs.json"), "w") as f:
            json.dump(known, f, indent=1)
        write_reference_graphs()
    write_formats(np.random.default_rng(20261204))
    write_ewise(np.random.default_rng(20261205))
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    if sys.argv[1:] in (["formats"], ["ewise"], ["graphs"]):
        if oracle.build_ref() is None:
            raise SystemExit("reference sources not available; cannot regenerate fixtures")
        if sys.argv[1] == "formats":
            print(write_formats(np.random.default_rng(20261204)))
        elif sys.argv[1] == "graphs":
            print(write_reference_graphs())
        else:
            print(write_ewise(np.random.default_rng(20261205)))
    else:
        main()
