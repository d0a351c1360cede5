"""The CUDA path against the golden fixtures made from the unmodified
reference (tests/golden/make_golden.py): bit-exact TC, per-row counts,
k-truss edge sets and iteration counts, masked products of every variant and
complemented-mask products; BC within 1e-9 (FP64)."""
import json
import os

import numpy as np
import pytest

import graphalgo_gb300 as ga

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def gold():
    data = np.load(os.path.join(GOLD, "synthetic.npz"))
    with open(os.path.join(GOLD, "synthetic.json")) as f:
        meta = json.load(f)
    return data, meta


def _dev(ctx, data, key):
    rst = data[key + "_rst"]
    m = len(rst) - 1
    return ga.Csr.upload(ctx, m, m, rst, data[key + "_col"], data[key + "_val"])


@pytest.mark.parametrize("algo", ["tri", "hybrid", "dot", "msa", "mca", "heap", "naive"])
def test_golden_tc(ctx, gold, algo):
    data, meta = gold
    for name, info in meta["graphs"].items():
        total, rows = ga.tc(algo, _dev(ctx, data, f"{name}_A"))
        assert total == info["triangles"], name
        assert np.array_equal(rows, data[f"{name}_tc_rows"]), name


@pytest.mark.parametrize("algo", ["tri", "hybrid", "dot", "msa", "mca", "heap", "naive"])
def test_golden_ktruss(ctx, gold, algo):
    data, meta = gold
    for name, info in meta["graphs"].items():
        G = _dev(ctx, data, f"{name}_A")
        for kt in info["ktruss"]:
            C, it = ga.ktruss(algo, G, kt["k"])
            r, c, v = C.download()
            key = f"{name}_k{kt['k']}"
            assert it == kt["iters"], (name, kt)
            assert np.array_equal(r, data[key + "_rst"]) and np.array_equal(c, data[key + "_col"]), (name, kt)
            assert np.array_equal(v, data[key + "_val"]), (name, kt)


def test_golden_square_and_bc(ctx, gold):
    data, meta = gold
    for name, info in meta["graphs"].items():
        G = _dev(ctx, data, f"{name}_A")
        for algo in ("msa", "mca", "heap", "naive", "dot", "hybrid", "tri"):
            assert np.array_equal(ga.mxm_masked(algo, G, G, G).download()[2], data[f"{name}_sq_val"]), (name, algo)
        ref = data[f"{name}_bc_f64"]
        got = ga.bc(G, data[f"{name}_bc_sources"])
        assert np.all(np.abs(got - ref) <= 1e-9 * np.maximum(np.abs(ref), 1.0)), name


def test_golden_mxm_and_cmask(ctx, gold):
    data, meta = gold
    for key in meta["mxm"]:
        A, B, M = (_dev(ctx, data, f"{key}_{x}") for x in "ABM")
        for algo in range(4):
            got = ga.mxm_masked(algo, A, B, M).download()[2]
            ref = data[f"{key}_algo{algo}_val"]
            if key.endswith("i32"):
                assert np.array_equal(got, ref), (key, algo)
            else:
                assert np.allclose(got, ref, rtol=1e-12, atol=1e-12), (key, algo)
        r, c, v = ga.mxm_cmask(A, B, M).download()
        assert np.array_equal(r, data[f"{key}_cmask_rst"]) and np.array_equal(c, data[f"{key}_cmask_col"])
        if key.endswith("i32"):
            assert np.array_equal(v, data[f"{key}_cmask_val"])
        else:
            assert np.allclose(v, data[f"{key}_cmask_val"], rtol=1e-12, atol=1e-12)
