"""Request server: results in the mix equal results alone, admission by the
HBM bound, refusal of requests that can never fit, and the byte bounds
against the allocations the calls actually make.

TC counts and k-truss edge sets / iteration counts are bit-exact; BC scores
within 1e-9 relative (absolute floor 1e-9).
"""
import numpy as np
import pytest

import graphalgo_gb300 as ga
from graphs import csr_from_arrays, to_device

pytestmark = pytest.mark.gpu

BC_RTOL = 1e-9


def _pool():
    g = [ga.gen_rmat(s, 16, seed=30 + s) for s in (8, 9, 10, 11, 12)]
    g += [ga.gen_knn(n, d, 30, seed=n + d) for n, d in ((300, 4), (800, 8), (1500, 12))]
    g += [ga.gen_er(2000, 12000, seed=5)]
    return g


POOL = _pool()


def _requests(count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        gid = int(rng.integers(len(POOL)))
        t = int(rng.integers(3))
        m = POOL[gid][0]
        if t == ga.REQ_BC:
            out.append((t, gid, 0, rng.choice(m, min(32, m), replace=False).astype(np.int32)))
        elif t == ga.REQ_KTRUSS:
            out.append((t, gid, int(rng.integers(3, 9)), None))
        else:
            out.append((t, gid, 0, None))
    return out


def _serve(server, reqs, gap=None):
    import time
    ids = []
    for i, (t, g, k, src) in enumerate(reqs):
        ids.append(server.submit(t, g, k=k, sources=src, want_edges=(t == ga.REQ_KTRUSS)))
        if gap:
            time.sleep(gap)
    return [server.wait(r, timeout=300) for r in ids]


def _same(a, b, t):
    assert a["status"] == ga.OK and b["status"] == ga.OK, (a.get("error"), b.get("error"))
    if t == ga.REQ_TC:
        assert a["tc"] == b["tc"]
    elif t == ga.REQ_KTRUSS:
        assert a["iters"] == b["iters"] and a["nnz"] == b["nnz"]
        assert np.array_equal(a["rst"], b["rst"]) and np.array_equal(a["col"], b["col"])
    else:
        np.testing.assert_allclose(a["bc"], b["bc"], rtol=BC_RTOL, atol=1e-9)


def _server(**kw):
    s = ga.Server(0, **kw)
    for m, rst, col in POOL:
        s.add_graph(m, rst, col)
    return s


def test_mix_equals_alone(built):
    reqs = _requests(90, seed=1)
    # alone: one worker, no batching, one request at a time
    with _server(workers=1, coalesce=False) as plain:
        alone = []
        for r in reqs:
            alone.extend(_serve(plain, [r]))
        assert all(a["batch_size"] == 1 for a in alone)
    # mix: every request queued at once, four workers, batching on
    with _server(workers=4, coalesce=True) as srv:
        mixed = _serve(srv, reqs)
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["rejected"] == 0
    assert st["batched_calls"] >= 1 and st["max_in_flight"] >= 2
    for (t, _, _, _), a, b in zip(reqs, alone, mixed):
        _same(a, b, t)


def test_results_match_direct_calls(ctx):
    reqs = _requests(24, seed=2)
    with _server(workers=3, coalesce=True) as srv:
        got = _serve(srv, reqs, gap=0.002)
    for (t, g, k, src), r in zip(reqs, got):
        m, rst, col = POOL[g]
        A = to_device(ctx, csr_from_arrays(m, rst, col))
        if t == ga.REQ_TC:
            assert r["tc"] == ga.tc("msa", A, per_row=False)[0]
        elif t == ga.REQ_KTRUSS:
            C, it = ga.ktruss("msa", A, k)
            cr, cc, _ = C.download()
            assert r["iters"] == it and np.array_equal(r["rst"], cr) and np.array_equal(r["col"], cc)
        else:
            np.testing.assert_allclose(r["bc"], ga.bc(A, src), rtol=BC_RTOL, atol=1e-9)


def test_admission_budget(built):
    """A budget that fits one large call at a time: calls never hold more
    than the budget, and a request whose bound exceeds it is refused."""
    m, rst, col = POOL[4]  # R-MAT scale 12
    nnz = len(col)
    b_kt = ga.request_bytes_bound(ga.REQ_KTRUSS, m, nnz)
    b_bc = ga.request_bytes_bound(ga.REQ_BC, m, nnz, 32)
    # the resident graph comes out of the budget
    budget = max(b_kt, b_bc) + 4 * (m + 1) + 8 * nnz + 1024
    with ga.Server(0, workers=4, coalesce=False, hbm_budget=budget) as srv:
        g = srv.add_graph(m, rst, col)
        ids = [srv.submit(ga.REQ_KTRUSS, g, k=4) for _ in range(6)]
        ids += [srv.submit(ga.REQ_BC, g, sources=np.arange(32, dtype=np.int32)) for _ in range(3)]
        big = srv.submit(ga.REQ_BC, g, sources=np.arange(m, dtype=np.int32))  # bound far above the budget
        res = [srv.wait(r, timeout=300) for r in ids]
        refused = srv.wait(big, timeout=300)
        st = srv.stats()
    assert all(r["status"] == ga.OK for r in res)
    assert refused["status"] == ga.ERR_ADMISSION
    assert st["rejected"] == 1
    assert st["peak_reserved"] <= st["budget"]
    assert st["max_in_flight"] == 1  # no two of these calls fit together


@pytest.mark.parametrize("gid", [2, 4, 6, 8])
def test_bounds_cover_allocations(ctx, gid):
    m, rst, col = POOL[gid]
    nnz = len(col)
    A = to_device(ctx, csr_from_arrays(m, rst, col))
    src = np.arange(min(32, m), dtype=np.int32)
    for t, run in ((ga.REQ_TC, lambda: ga.tc("msa", A, per_row=False)),
                   (ga.REQ_TC, lambda: ga.tc("dot", A, per_row=False)),
                   (ga.REQ_TC, lambda: ga.tc("tri", A, per_row=False)),
                   (ga.REQ_KTRUSS, lambda: ga.ktruss("msa", A, 4)),
                   (ga.REQ_KTRUSS, lambda: ga.ktruss("tri", A, 4)),
                   (ga.REQ_BC, lambda: ga.bc(A, src))):
        ctx.sync()
        base, _ = ctx.mem_stats(reset_peak=True)
        out = run()
        del out
        _, peak = ctx.mem_stats()
        bound = ga.request_bytes_bound(t, m, nnz, len(src))
        assert peak - base <= bound, (t, peak - base, bound)


def test_concurrent_bc_with_different_source_counts(built):
    """Two host threads, each with its own context, run BC with 8 and with
    300 sources at the same time: the forward kernel's shared-memory size
    differs per call, and no call may fail because of the other."""
    from concurrent.futures import ThreadPoolExecutor
    m, rst, col = ga.gen_rmat(11, 16, seed=91)
    rng = np.random.default_rng(3)
    sets = [rng.choice(m, 8, replace=False).astype(np.int32), rng.choice(m, 300, replace=False).astype(np.int32)]
    refs = []
    with ga.Context(0) as c0:
        A0 = ga.Csr.upload(c0, m, m, rst, col)
        refs = [ga.bc(A0, s) for s in sets]
        A0.free()

    def run(which):
        with ga.Context(0) as c:
            A = ga.Csr.upload(c, m, m, rst, col)
            out = [ga.bc(A, sets[which]) for _ in range(12)]
            A.free()
            return out

    with ThreadPoolExecutor(2) as ex:
        futs = [ex.submit(run, w) for w in (0, 1)]
        results = [f.result() for f in futs]
    for w in (0, 1):
        for got in results[w]:
            np.testing.assert_allclose(got, refs[w], rtol=BC_RTOL, atol=1e-9)


def test_pool_from_device_and_files(ctx, tmp_path):
    """Graphs added from a device CSR or from a graph file serve the same
    results as the same graph uploaded from the host."""
    scale = 9
    m, rst, col = ga.gen_rmat(scale, 16, seed=77)
    D = ga.gen_rmat_device(ctx, scale, 16, seed=77)
    # a Matrix Market file holding the lower triangle, as the reference's graphs do
    lo = [(i, j) for i in range(m) for j in col[rst[i]:rst[i + 1]] if j < i]
    mtx = tmp_path / "g.mtx"
    with open(mtx, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern symmetric\n")
        f.write(f"{m} {m} {len(lo)}\n")
        f.writelines(f"{i + 1} {j + 1}\n" for i, j in lo)
    binp = tmp_path / "g.bin"
    ga.write_bin(D, str(binp))
    with ga.Server(0, workers=2, coalesce=True) as srv:
        g_host = srv.add_graph(m, rst, col)
        g_dev = srv.add_graph_device(D)
        g_mtx = srv.add_graph_file(str(mtx))
        g_bin = srv.add_graph_file(str(binp))
        assert srv.sizes == [m] * 4
        with pytest.raises(ga.GaError):
            srv.add_graph_file(str(tmp_path / "g.txt"))
        src = np.arange(0, m, m // 16, dtype=np.int32)[:16]
        reqs = [(t, g, k, s) for g in (g_host, g_dev, g_mtx, g_bin)
                for t, k, s in ((ga.REQ_TC, 0, None), (ga.REQ_KTRUSS, 4, None), (ga.REQ_BC, 0, src))]
        got = _serve(srv, reqs)
    for i in range(3):
        for j in (1, 2, 3):
            _same(got[i], got[3 * j + i], reqs[i][0])
    assert got[0]["tc"] > 0


def test_cancel_queued_requests(built):
    """Requests still queued behind a busy single worker can be cancelled:
    they complete with GA_ERR_CANCELLED; the others run normally."""
    with ga.Server(0, workers=1, coalesce=False) as srv:
        for m, rst, col in POOL:
            srv.add_graph(m, rst, col)
        big = len(POOL) - 5  # rmat12
        m = POOL[big][0]
        first = [srv.submit(ga.REQ_BC, big, sources=np.arange(min(256, m), dtype=np.int32)),
                 srv.submit(ga.REQ_KTRUSS, big, k=3)]
        rest = [srv.submit(ga.REQ_TC, g % len(POOL)) for g in range(20)]
        cancelled = {rid: srv.cancel(rid) for rid in reversed(rest)}
        assert any(cancelled.values())
        for rid in first:
            assert srv.wait(rid)["status"] == ga.OK
        for rid in rest:
            r = srv.wait(rid)
            if cancelled[rid]:
                assert r["status"] == ga.ERR_CANCELLED and r["error"]
            else:
                assert r["status"] == ga.OK and r["tc"] >= 0
        st = srv.stats()
        assert st["cancelled"] == sum(cancelled.values())
        # a finished request cannot be cancelled
        done = srv.submit(ga.REQ_TC, 0)
        srv.wait(done, release=False)
        assert srv.cancel(done) is False
