"""CPU checks of the host-side logic around the kernels: the request server's
argument handling and byte bounds, and the benchmark's seeded workloads."""
import ctypes
import os
import sys

import numpy as np
import pytest

import graphalgo_gb300 as ga

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_request_bounds_grow_with_the_work(built):
    kt = [ga.request_bytes_bound(ga.REQ_KTRUSS, 1000, z) for z in (0, 10_000, 100_000)]
    assert kt[0] < kt[1] < kt[2]
    tc = [ga.request_bytes_bound(ga.REQ_TC, m, 50_000) for m in (100, 10_000)]
    assert tc[0] < tc[1]
    bc = [ga.request_bytes_bound(ga.REQ_BC, 10_000, 50_000, ns) for ns in (1, 32, 256)]
    assert bc[0] < bc[1] < bc[2]
    # BC keeps per (vertex, source) state: at least 40 bytes per pair
    assert bc[2] >= 40 * 10_000 * 256


def test_request_bounds_reject_bad_arguments(built):
    L = ga.lib()
    out = ctypes.c_int64()
    assert L.ga_request_bytes_bound(ctypes.c_int(7), ctypes.c_int64(10), ctypes.c_int64(10), ctypes.c_int64(0),
                                    ctypes.byref(out)) == ga.ERR_INVALID_ARG
    assert L.ga_request_bytes_bound(ctypes.c_int(ga.REQ_TC), ctypes.c_int64(-1), ctypes.c_int64(10),
                                    ctypes.c_int64(0), ctypes.byref(out)) == ga.ERR_INVALID_ARG
    assert L.ga_request_bytes_bound(ctypes.c_int(ga.REQ_TC), ctypes.c_int64(1), ctypes.c_int64(1),
                                    ctypes.c_int64(0), None) == ga.ERR_INVALID_ARG


def test_server_entry_points_reject_null_handles(built):
    L = ga.lib()
    res = ga.ServerResult()
    rid = ctypes.c_int64()
    gid = ctypes.c_int()
    assert L.ga_server_create(ctypes.c_int(0), None, None) == ga.ERR_INVALID_ARG
    assert L.ga_server_submit(None, ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0), None, ctypes.c_int(0),
                              ctypes.c_int(0), ctypes.byref(rid)) == ga.ERR_INVALID_ARG
    assert L.ga_server_wait(None, ctypes.c_int64(1), ctypes.c_double(0.1), ctypes.byref(res)) == ga.ERR_INVALID_ARG
    assert L.ga_server_release(None, ctypes.c_int64(1)) == ga.ERR_INVALID_ARG
    assert L.ga_server_drain(None, ctypes.c_double(0.1)) == ga.ERR_INVALID_ARG
    assert L.ga_server_destroy(None) == ga.ERR_INVALID_ARG
    assert L.ga_server_add_graph(None, ctypes.c_int64(1), None, None, ctypes.byref(gid)) == ga.ERR_INVALID_ARG
    stats = ga.ServerStats()
    assert L.ga_server_get_stats(None, ctypes.byref(stats)) == ga.ERR_INVALID_ARG


def test_batch_entry_points_reject_null_handles(built):
    L = ga.lib()
    v = np.zeros(2, np.int64)
    assert L.ga_batch_tc(None, ctypes.c_int(0), None, ctypes.c_int64(1), v.ctypes.data_as(ctypes.c_void_p),
                         None) == ga.ERR_INVALID_ARG
    assert L.ga_batch_bc(None, None, ctypes.c_int64(1), None, None, None, None) == ga.ERR_INVALID_ARG
    assert L.ga_csr_block_diag(None, ctypes.c_int64(0), None, None, None) == ga.ERR_INVALID_ARG


def test_bench_workloads_are_seeded():
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    n1, d1 = bench.knn_batch_sizes(4096, 42)
    n2, d2 = bench.knn_batch_sizes(4096, 42)
    assert np.array_equal(n1, n2) and np.array_equal(d1, d2)
    assert n1.min() >= 32 and n1.max() <= 4096 and d1.min() >= 4 and d1.max() <= 16

    class Args:
        seed = 42
    pool = [("g%d" % i, 100 + i, None, None) for i in range(11)]
    reqs = bench.serve_requests(Args, pool, 300)
    assert len(reqs) == 300
    again = bench.serve_requests(Args, pool, 300)
    assert all(a[:3] == b[:3] for a, b in zip(reqs, again))
    types = np.bincount([r[0] for r in reqs], minlength=3)
    assert types.min() > 60  # uniform over TC / k-truss / BC
    for t, g, k, src in reqs:
        if t == ga.REQ_KTRUSS:
            assert 3 <= k <= 8
        if t == ga.REQ_BC:
            m = pool[g][1]
            assert len(src) == 32 and len(set(src.tolist())) == 32 and src.max() < m


def test_tune_cache_file_round_trip(built, tmp_path):
    """The tuning cache file: entries load, save back unchanged, a malformed
    file loads nothing, clear empties the cache (no GPU involved)."""
    src = tmp_path / "tune.txt"
    lines = ["ga_tune 1 0 0 37 37 47 0 0 2 -1  7 32768 1048576 0 8 16 0 2.5 9.25 14",
             "ga_tune 1 0 2 25 25 35 0 0 2 -1  4 32768 1048576 0 8 16 1 0.019 0.07 7"]
    src.write_text("\n".join(lines) + "\n")
    ga.tune_clear()
    assert ga.tune_load(str(src)) == 2
    out = tmp_path / "saved.txt"
    assert ga.tune_save(str(out)) == 2
    saved = sorted(" ".join(l.split()) for l in out.read_text().splitlines())
    assert saved == sorted(" ".join(l.split()) for l in lines)
    bad = tmp_path / "bad.txt"
    bad.write_text(lines[0] + "\nga_tune 1 0 0 1 1 1 0 0 2 -1 5 0 0 0 8 16 0 1 1 1\n")  # GA_AUTO is no choice
    with pytest.raises(ga.GaError):
        ga.tune_load(str(bad))
    with pytest.raises(ga.GaError):
        ga.tune_load(str(tmp_path / "missing.txt"))
    ga.tune_clear()
    assert ga.tune_save(str(out)) == 0


def test_server_cancel_rejects_null_server(built):
    assert ga.lib().ga_server_cancel(None, ctypes.c_int64(1)) == ga.ERR_INVALID_ARG


@pytest.mark.parametrize("scale,ef,seed", [(6, 4, 1), (12, 16, 4), (16, 16, 42)])
def test_oracle_rmat_generator_matches_the_product(built, scale, ef, seed):
    """The oracle side's R-MAT generator (oracle/gen.c, used by the reference
    arm of bench.py so it never loads the product's library) gives the
    product's graph bit for bit."""
    import oracle
    m, rst, col = ga.gen_rmat(scale, ef, 0.57, 0.19, 0.19, seed)
    om, orst, ocol = oracle.gen_rmat(scale, ef, 0.57, 0.19, 0.19, seed)
    assert om == m and np.array_equal(orst, rst) and np.array_equal(ocol, col)
