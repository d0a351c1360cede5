"""Autotuner and schedule options: every schedule and every tuned choice
gives the same (bit-exact) results; tuning is cached per problem signature
and leaves the work counters untouched."""
import numpy as np
import pytest

import graphalgo_gb300 as ga
import oracle
from graphs import csr_from_arrays, random_csr, to_device

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rmat(ctx):
    G = csr_from_arrays(*ga.gen_rmat(11, 16, seed=77))
    return G, to_device(ctx, G)


def test_autotune_ktruss_cached_and_exact(ctx, rmat):
    G, A = rmat
    before = ctx.work_counters()
    r1 = ga.autotune(ga.TUNE_KTRUSS, A, force=True)
    assert r1["algo"] in ("msa", "mca", "dot", "hybrid", "tri") and r1["cached"] == 0 and r1["candidates"] >= 5
    assert 0 < r1["ms"] <= r1["default_ms"] + 1e-9
    r2 = ga.autotune(ga.TUNE_KTRUSS, A)
    assert r2["cached"] == 1 and r2["algo"] == r1["algo"]
    assert ctx.work_counters() == before, "tuning launches are not counted"
    for k in (3, 5):
        R, it = oracle.ktruss(G, k)
        C, git = ga.ktruss("auto", A, k)
        r, c, _ = C.download()
        assert git == it and np.array_equal(r, R.rst) and np.array_equal(c, R.col)


def test_autotune_tc_and_product(ctx, rmat):
    G, A = rmat
    r = ga.autotune(ga.TUNE_TC, A, force=True)
    assert r["algo"] in ("msa", "mca", "dot", "tri")
    assert ga.tc("auto", A, per_row=False)[0] == oracle.tc_sandia(G)[0]
    rng = np.random.default_rng(8)
    X = random_csr(300, 200, 0.05, rng)
    Y = random_csr(200, 250, 0.05, rng)
    Mk = random_csr(300, 250, 0.2, rng)
    Xd, Yd, Md = to_device(ctx, X), to_device(ctx, Y), to_device(ctx, Mk)
    r = ga.autotune(ga.TUNE_PRODUCT, Xd, Yd, Md, force=True)
    assert r["candidates"] >= 5
    got = ga.mxm_masked("auto", Xd, Yd, Md).download()[2]
    assert np.array_equal(got, oracle.mxm_masked(X, Y, Mk))


@pytest.mark.parametrize("opt,val", [(ga.OPT_MXM_WARP_FLOPS, 0), (ga.OPT_MXM_WARP_FLOPS, 1 << 40),
                                     (ga.OPT_MXM_HEAVY_FLOPS, 1), (ga.OPT_MXM_CTAS_PER_SM, 1),
                                     (ga.OPT_DOT_CHUNK, 1), (ga.OPT_DOT_CHUNK, 64),
                                     (ga.OPT_HYBRID_RATIO, 0), (ga.OPT_HYBRID_RATIO, 1 << 20),
                                     (ga.OPT_TRI_ORDER, 1)])
def test_schedule_options_do_not_change_results(ctx, rmat, opt, val):
    G, A = rmat
    ref = oracle.mxm_masked(G, G, G)
    defaults = {ga.OPT_MXM_WARP_FLOPS: 32768, ga.OPT_MXM_HEAVY_FLOPS: 1 << 20, ga.OPT_MXM_CTAS_PER_SM: 0,
                ga.OPT_DOT_CHUNK: 8, ga.OPT_HYBRID_RATIO: 16, ga.OPT_TRI_ORDER: 0}
    ctx.set_option(opt, val)
    try:
        for algo in ("msa", "mca", "heap", "dot", "hybrid", "tri"):
            assert np.array_equal(ga.mxm_masked(algo, A, A, A).download()[2], ref), algo
        R, rit = oracle.ktruss(G, 4)
        for algo in ("msa", "tri"):
            C, it = ga.ktruss(algo, A, 4)
            assert it == rit and np.array_equal(C.download()[1], R.col), algo
        assert ga.tc("tri", A, per_row=False)[0] == oracle.tc_sandia(G)[0]
    finally:
        ctx.set_option(opt, defaults[opt])


def test_bad_options_rejected(ctx):
    for opt, val in ((ga.OPT_DOT_CHUNK, 0), (ga.OPT_MXM_CTAS_PER_SM, -1), (ga.OPT_TRI_ORDER, 2), (99, 1)):
        with pytest.raises(ga.GaError):
            ctx.set_option(opt, val)


def test_batch_auto(ctx):
    n = np.array([50, 700, 2000, 300], np.int32)
    U, voff = ga.gen_knn_batch(ctx, n, np.array([4, 8, 12, 16], np.int32), k=30, seed=5)
    t_auto = ga.batch_tc("auto", U, voff)
    t_msa = ga.batch_tc("msa", U, voff)
    assert np.array_equal(t_auto, t_msa)
    Ca, ia = ga.batch_ktruss("auto", U, voff, 4)
    Cm, im = ga.batch_ktruss("msa", U, voff, 4)
    assert np.array_equal(ia, im)
    assert all(np.array_equal(x, y) for x, y in zip(Ca.download(), Cm.download()))


def test_tune_cache_file_restores_choices(ctx, rmat, tmp_path):
    """A saved cache, loaded into a cleared process cache, answers GA_AUTO
    without re-tuning and with the same choice."""
    G, A = rmat
    r1 = ga.autotune(ga.TUNE_KTRUSS, A, force=True)
    path = str(tmp_path / "tune.txt")
    assert ga.tune_save(path) >= 1
    ga.tune_clear()
    assert ga.tune_load(path) >= 1
    r2 = ga.autotune(ga.TUNE_KTRUSS, A)
    assert r2["cached"] == 1 and r2["algo"] == r1["algo"] and r2["tri_order"] == r1["tri_order"]
    R, it = oracle.ktruss(G, 4)
    C, git = ga.ktruss("auto", A, 4)
    assert git == it and np.array_equal(C.download()[1], R.col)
