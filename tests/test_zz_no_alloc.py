"""The allocation-free masked product, ga_mxm_masked_noalloc.

It serves callers that cannot allocate device memory when they need the
product (applications that keep all device memory in their own arena,
latency-critical callers that cannot accept the device synchronisation of
cudaMalloc / cudaFree): they pass device buffers for everything and the
kernel's scratch lives in a fixed array inside the library. These
tests call it through the C ABI twice in a row, on the same shared scratch,
and inside a captured CUDA graph, and compare each result with the
allocating entry point's (ga_mxm_masked), exactly - the values are integers.
"""
import ctypes

import numpy as np
import pytest

import graphalgo_gb300 as ga

pytestmark = pytest.mark.gpu

_p = ctypes.c_void_p
_i64 = ctypes.c_int64


def _noalloc(stream, algo, m, k, n, A, B, M, mask_nnz, dtype, b_unit, c_ptr):
    f = ga.lib().ga_mxm_masked_noalloc
    f.restype = ctypes.c_int
    ar, ac, av = A.device_ptrs()
    br, bc, bv = B.device_ptrs()
    mr, mc, _ = M.device_ptrs()
    return f(_p(stream), int(algo), _i64(m), _i64(k), _i64(n), _p(ar), _p(ac), _p(av), _p(br), _p(bc), _p(bv),
             _p(mr), _p(mc), _i64(mask_nnz), int(dtype), int(b_unit), _p(c_ptr))


def _dense_ptr(D):
    v = _p()
    assert ga.lib().ga_dense_device_ptr(D.handle, ctypes.byref(v)) == 0
    return int(v.value)


@pytest.mark.parametrize("algo,unit", [(ga.MSA, True), (ga.MSA, False), (ga.MCA, False), (ga.HEAP, False)])
def test_noalloc_matches_allocating_entry_point(ctx, algo, unit):
    m, rst, col = ga.gen_rmat(12, 16, seed=31)
    rng = np.random.default_rng(4)
    vals = np.ones(len(col), np.int32) if unit else rng.integers(-3, 4, len(col)).astype(np.int32)
    A = ga.Csr.upload(ctx, m, m, rst, col, vals)
    # a different mask: every other entry of A's pattern
    keep = np.zeros(len(col), bool)
    keep[::2] = True
    mrow = np.repeat(np.arange(m), np.diff(rst))[keep]
    mrst = np.zeros(m + 1, np.int32)
    np.add.at(mrst, mrow + 1, 1)
    mrst = np.cumsum(mrst).astype(np.int32)
    M = ga.Csr.upload(ctx, m, m, mrst, col[keep])
    nnz = M.nnz
    expected = ga.mxm_masked(algo, A, A, M).download()[2]
    out = ga.Dense.create(ctx, 1, nnz, ga.INT32, np.full(nnz, -7, np.int32))
    stream = ctx.stream()
    for call in range(2):
        rc = _noalloc(stream, algo, m, m, m, A, A, M, nnz, ga.INT32, 1 if unit else 0, _dense_ptr(out))
        assert rc == ga.OK, (call, rc)
        ctx.sync()
        got = out.download().ravel()
        assert np.array_equal(got, expected), call


def test_noalloc_rejects_shapes_beyond_its_scratch(ctx):
    m, rst, col = ga.gen_er(100, 300, seed=2)
    A = ga.Csr.upload(ctx, m, m, rst, col)
    out = ga.Dense.create(ctx, 1, A.nnz, ga.INT32)
    # claims 50M rows: the scratch this needs exceeds the fixed array, so the
    # call is refused before anything is launched
    rc = _noalloc(ctx.stream(), ga.MSA, 50_000_000, m, m, A, A, A, A.nnz, ga.INT32, 1, _dense_ptr(out))
    assert rc == ga.ERR_INVALID_ARG
    rc = _noalloc(ctx.stream(), ga.NAIVE, m, m, m, A, A, A, A.nnz, ga.INT32, 1, _dense_ptr(out))
    assert rc == ga.ERR_UNSUPPORTED


def test_noalloc_rejects_missing_arrays(ctx):
    """Refused before any launch: the sorted merge reads B's values even when
    they are all 1, so GA_HEAP with b_unit set still needs b_val; the column
    arrays are always needed."""
    m, rst, col = ga.gen_er(100, 300, seed=2)
    A = ga.Csr.upload(ctx, m, m, rst, col)
    out = _dense_ptr(ga.Dense.create(ctx, 1, A.nnz, ga.INT32))
    f = ga.lib().ga_mxm_masked_noalloc
    f.restype = ctypes.c_int
    ar, ac, av = A.device_ptrs()

    def call(algo, a_col, b_col, b_val):
        return f(_p(ctx.stream()), int(algo), _i64(m), _i64(m), _i64(m), _p(ar), _p(a_col), _p(av), _p(ar),
                 _p(b_col), _p(b_val), _p(ar), _p(ac), _i64(A.nnz), int(ga.INT32), 1, _p(out))

    assert call(ga.HEAP, ac, ac, None) == ga.ERR_INVALID_ARG
    assert call(ga.MSA, None, ac, av) == ga.ERR_INVALID_ARG
    assert call(ga.MSA, ac, None, av) == ga.ERR_INVALID_ARG


def test_noalloc_captured_in_a_cuda_graph(ctx):
    """After one eager call (the per-device setup), the call is captured into
    a CUDA graph on a caller's stream (nothing in it allocates or
    synchronises, which capture refuses); the graph, replayed twice into an
    output reset before each replay, gives ga_mxm_masked's values."""
    torch = pytest.importorskip("torch")
    m, rst, col = ga.gen_rmat(11, 16, seed=33)
    A = ga.Csr.upload(ctx, m, m, rst, col)
    expected = ga.mxm_masked(ga.MSA, A, A, A).download()[2]
    nnz = A.nnz
    out = torch.full((nnz,), -7, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    ctx.sync()
    torch.cuda.synchronize()
    assert _noalloc(s.cuda_stream, ga.MSA, m, m, m, A, A, A, nnz, ga.INT32, 1, out.data_ptr()) == ga.OK
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), expected)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        rc = _noalloc(s.cuda_stream, ga.MSA, m, m, m, A, A, A, nnz, ga.INT32, 1, out.data_ptr())
    assert rc == ga.OK
    for _ in range(2):
        out.fill_(-7)
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), expected)
