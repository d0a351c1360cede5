#!/usr/bin/env python3
"""Golden record of the benchmark's k-truss sweep, made by the CPU oracle.

The sweep: R-MAT scale 18, edge factor 16, a/b/c = 0.57/0.19/0.19, seed 42
(made by oracle.gen_rmat, the same graph as the product's generator), then
C_3 = k_truss(A, 3) and C_k = k_truss(C_{k-1}, k) until the truss is empty
(src/main.cpp:90-146, restated by oracle.ktruss). For every k the record
holds the iteration count the reference prints, the number of stored
entries, and a BLAKE2b digest of the edge set (row starts then columns, as
little-endian int32 bytes). Where the reference library was built here
(oracle/_ref), the first stages are also run through the reference's own
k_truss and must agree.

bench.py compares the GPU sweep's every k-truss with this record; the -m gpu
tests compare a smaller sweep with the oracle live.

    python tests/golden/make_sweep.py            # writes rmat18_sweep.json
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

SCALE, EF, SEED = 18, 16, 42
REF_STAGES = 2  # stages also run through the unmodified reference


def edge_digest(rst: np.ndarray, col: np.ndarray) -> str:
    h = hashlib.blake2b(digest_size=16)
    h.update(np.ascontiguousarray(rst, "<i4").tobytes())
    h.update(np.ascontiguousarray(col, "<i4").tobytes())
    return h.hexdigest()


def main():
    oracle.build()
    oracle.set_num_threads(os.cpu_count() or 1)
    m, rst, col = oracle.gen_rmat(SCALE, EF, 0.57, 0.19, 0.19, SEED)
    A = oracle.Csr(m, m, rst, col, np.ones(len(col), np.int32))
    rec = {"graph": {"scale": SCALE, "edge_factor": EF, "abc": [0.57, 0.19, 0.19], "seed": SEED, "vertices": m,
                     "stored_entries": int(len(col)), "digest": edge_digest(rst, col)},
           "digest": "blake2b-128 over little-endian int32 row starts, then columns", "stages": []}
    ref = oracle.build_ref() is not None
    cur, k = A, 3
    t0 = time.time()
    while True:
        C, it = oracle.ktruss(cur, k)
        if ref and len(rec["stages"]) < REF_STAGES:
            R, rit = oracle.ref_ktruss(cur, k)
            assert rit == it and np.array_equal(R.rst, C.rst) and np.array_equal(R.col, C.col), k
        rec["stages"].append([k, int(it), int(C.nnz), edge_digest(C.rst, C.col)])
        print(f"k={k} iters={it} nnz={C.nnz} ({time.time() - t0:.1f} s)", flush=True)
        if C.nnz == 0:
            break
        cur, k = C, k + 1
    rec["reference_checked_stages"] = REF_STAGES if ref else 0
    with open(os.path.join(HERE, "rmat18_sweep.json"), "w") as f:
        json.dump(rec, f, indent=0)


if __name__ == "__main__":
    main()
