"""CPU checks of the shipped library: it loads, exports every entry point the
header declares, reports errors through status codes without a GPU, and its
seeded generators produce well-formed symmetric CSR."""
import ctypes
import os
import re

import numpy as np
import pytest

import graphalgo_gb300 as ga

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    with open(os.path.join(ROOT, "include", "graphalgo_gb300.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"GA_API[^;(]*?\b(ga_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    L = ga.lib()
    names = declared_symbols()
    assert len(names) >= 50
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings(built):
    L = ga.lib()
    assert L.ga_status_string(ga.OK) == b"ok"
    assert L.ga_status_string(ga.ERR_INVALID_CSR) == b"invalid CSR"


@pytest.mark.skipif(ga.device_count() > 0 if os.path.exists(ga.LIB_PATH) else False,
                    reason="a CUDA device is present")
def test_context_fails_loudly_without_device(built):
    with pytest.raises(ga.GaError) as e:
        ga.Context(0)
    assert e.value.code == ga.ERR_NO_DEVICE


def test_null_arguments_are_rejected(built):
    L = ga.lib()
    assert L.ga_ctx_create(0, None, None) == ga.ERR_INVALID_ARG
    assert L.ga_csr_free(None, None) == ga.ERR_INVALID_ARG
    assert L.ga_mxm_masked(None, 0, None, None, None, None) == ga.ERR_INVALID_ARG
    assert L.ga_ktruss_sweep_begin(None, 0, None, 3, None) == ga.ERR_INVALID_ARG
    assert L.ga_ktruss_sweep_next(None, None, None, None) == ga.ERR_INVALID_ARG
    assert L.ga_ktruss_sweep_free(None) == ga.OK
    assert L.ga_csr_set_symmetric(None, None, 1) == ga.ERR_INVALID_ARG


def _check_graph(m, rst, col):
    assert rst[0] == 0 and rst[-1] == len(col) and np.all(np.diff(rst) >= 0)
    rows = np.repeat(np.arange(m), np.diff(rst))
    assert np.all(col >= 0) and np.all(col < m)
    assert not np.any(rows == col), "self-loop"
    for i in range(0, m, max(1, m // 200)):
        seg = col[rst[i]:rst[i + 1]]
        assert np.all(np.diff(seg) > 0), "unsorted or duplicate"
    key = set(zip(rows.tolist(), col.tolist()))
    assert all((c, r) in key for r, c in list(key)[:2000]), "not symmetric"


def test_generators_deterministic_and_well_formed(built):
    a = ga.gen_rmat(10, 16, seed=5)
    b = ga.gen_rmat(10, 16, seed=5)
    c = ga.gen_rmat(10, 16, seed=6)
    assert np.array_equal(a[1], b[1]) and np.array_equal(a[2], b[2])
    assert not np.array_equal(a[2], c[2])
    _check_graph(*a)
    m, rst, col = ga.gen_er(1000, 9990, seed=7)
    assert m == 1000 and len(col) == 2 * 9990
    _check_graph(m, rst, col)
    m, rst, col = ga.gen_knn(300, 4, 10, seed=2)
    assert np.all(np.diff(rst) >= 10)
    _check_graph(m, rst, col)


def test_generator_argument_errors(built):
    L = ga.lib()
    m, z = ctypes.c_int64(), ctypes.c_int64()
    r, c = ctypes.c_void_p(), ctypes.c_void_p()
    assert L.ga_gen_er(10, 1000, 1, ctypes.byref(m), ctypes.byref(z), ctypes.byref(r), ctypes.byref(c)) \
        == ga.ERR_INVALID_ARG
    assert L.ga_gen_rmat(0, 16, ctypes.c_double(0.57), ctypes.c_double(0.19), ctypes.c_double(0.19), 1,
                         ctypes.byref(m), ctypes.byref(z), ctypes.byref(r), ctypes.byref(c)) == ga.ERR_INVALID_ARG
