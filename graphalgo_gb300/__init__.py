"""graphalgo_gb300: GB300-native masked SpGEMM C<M> = A*B over CSR graphs.

Python binding (ctypes) over the C ABI in ``include/graphalgo_gb300.h``;
the kernels live in ``graphalgo_gb300/_lib/libgraphalgo_gb300.so``, built
in-tree by ``graphalgo_gb300.build.build()``. There is no CPU fallback: if the
library is missing, ``lib()`` raises, and if no CUDA device is usable,
``Context()`` raises.

The entry points mirror the reference's (UAlex322/GraphAlgo) operator API:
``mxm_masked`` for mxmm_msa / mxmm_mca / mxmm_heap / mxmm_naive
(include/matrix_la.h:700-1277), ``mxm_cmask`` for mxmm_msa_cmask (788-891),
``mxm_spd`` (241-270), ``tc`` for triangle_counting_masked_sandia
(src/main.cpp:65-86), ``ktruss`` for k_truss (src/main.cpp:90-146) and ``bc``
for betweenness_centrality_batch (include/betweenness_centrality.h:125-237).
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgraphalgo_gb300.so")

# dtypes
INT32, INT64, FP32, FP64, UINT8 = 0, 1, 2, 3, 4
# algorithms
MSA, MCA, HEAP, NAIVE, DOT, AUTO, HYBRID, TRI = 0, 1, 2, 3, 4, 5, 6, 7
ALGOS = {"msa": MSA, "mca": MCA, "heap": HEAP, "naive": NAIVE, "dot": DOT, "auto": AUTO, "hybrid": HYBRID,
         "tri": TRI}
ALGO_NAMES = {v: k for k, v in ALGOS.items()}
# options
OPT_DEVICE_LOOPS, OPT_PROFILE, OPT_FAIL_ALLOC_AFTER, OPT_KNN_TILED = 1, 2, 3, 4
OPT_MXM_WARP_FLOPS, OPT_MXM_HEAVY_FLOPS, OPT_MXM_CTAS_PER_SM, OPT_DOT_CHUNK, OPT_HYBRID_RATIO = 5, 6, 7, 8, 9
OPT_TRI_ORDER, OPT_KT_FRONTIER = 10, 11
OPT_BC_BACKWARD = 12
TUNE_KTRUSS, TUNE_PRODUCT, TUNE_TC = 0, 1, 2
# edge-list / file ingestion flags
EDGES_MIRROR, EDGES_DROP_LOOPS, EDGES_LOWER_SYMM, EDGES_UNIT = 1, 2, 4, 8
# status codes
OK, ERR_INVALID_ARG, ERR_INVALID_CSR, ERR_SHAPE, ERR_DTYPE, ERR_CUDA, ERR_OOM, ERR_NO_DEVICE, \
    ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_ADMISSION, ERR_CANCELLED = range(12)

_NP = {INT32: np.int32, INT64: np.int64, FP32: np.float32, FP64: np.float64, UINT8: np.uint8}
_DT = {np.dtype(v): k for k, v in _NP.items()}

_i64 = ctypes.c_int64
_p = ctypes.c_void_p
_int = ctypes.c_int


class GaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 48), ("launches", ctypes.c_int64), ("total_ms", ctypes.c_double)]


_lib = None


def lib() -> ctypes.CDLL:
    """Load the CUDA library (raises when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with graphalgo_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    L.ga_last_error.restype = ctypes.c_char_p
    L.ga_status_string.restype = ctypes.c_char_p
    L.ga_host_free.restype = None
    for name in ("ga_gen_rmat",):
        getattr(L, name).argtypes = [_int, _int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_uint64, ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                                     ctypes.POINTER(_p), ctypes.POINTER(_p)]
    L.ga_gen_er.argtypes = [_i64, _i64, ctypes.c_uint64, ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                            ctypes.POINTER(_p), ctypes.POINTER(_p)]
    L.ga_gen_knn.argtypes = [_i64, _int, _int, ctypes.c_uint64, ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                             ctypes.POINTER(_p), ctypes.POINTER(_p)]
    L.ga_ctx_set_option.argtypes = [_p, _int, _i64]
    L.ga_gen_rmat_device.argtypes = [_p, _int, _int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_uint64, ctypes.POINTER(_p)]
    _lib = L
    return L


def device_count() -> int:
    c = _int(0)
    lib().ga_device_count(ctypes.byref(c))
    return int(c.value)


def _check(rc: int, ctx: Optional["Context"] = None):
    if rc != OK:
        L = lib()
        msg = L.ga_last_error(ctx.handle).decode() if ctx is not None and ctx.handle else ""
        if not msg:
            msg = L.ga_status_string(rc).decode()
        raise GaError(rc, msg)


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_p)


class Context:
    """One CUDA context handle (device, stream, memory pool)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        self.handle = _p()
        _check(lib().ga_ctx_create(int(device), _p(stream) if stream else None, ctypes.byref(self.handle)))

    def close(self):
        if self.handle:
            lib().ga_ctx_destroy(self.handle)
            self.handle = _p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        _check(lib().ga_ctx_sync(self.handle), self)

    def stream(self) -> int:
        s = _p()
        _check(lib().ga_ctx_stream(self.handle, ctypes.byref(s)), self)
        return int(s.value or 0)

    def set_option(self, option: int, value: int):
        _check(lib().ga_ctx_set_option(self.handle, int(option), int(value)), self)

    def timer_start(self):
        _check(lib().ga_timer_start(self.handle), self)

    def timer_stop(self) -> float:
        ms = ctypes.c_double()
        _check(lib().ga_timer_stop(self.handle, ctypes.byref(ms)), self)
        return float(ms.value)

    def kernel_stats(self) -> dict:
        n = _int()
        _check(lib().ga_ctx_kernel_stats(self.handle, None, 0, ctypes.byref(n)), self)
        arr = (KernelStat * max(1, n.value))()
        _check(lib().ga_ctx_kernel_stats(self.handle, arr, n.value, ctypes.byref(n)), self)
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(n.value)}

    def reset_kernel_stats(self):
        _check(lib().ga_ctx_reset_kernel_stats(self.handle), self)

    def mem_info(self) -> Tuple[int, int]:
        f, t = _i64(), _i64()
        _check(lib().ga_mem_info(self.handle, ctypes.byref(f), ctypes.byref(t)), self)
        return int(f.value), int(t.value)

    def mem_stats(self, reset_peak: bool = False) -> Tuple[int, int]:
        """(bytes held now, peak since the last reset) by this context's allocations."""
        u, p = _i64(), _i64()
        _check(lib().ga_ctx_mem_stats(self.handle, ctypes.byref(u), ctypes.byref(p), _int(int(reset_peak))), self)
        return int(u.value), int(p.value)

    def work_counters(self, reset: bool = False) -> dict:
        """Masked-SpGEMM work since the last reset: Gustavson products P of the
        requested products, mask entries, launches, A entries, rows, the
        products the Gustavson kernels processed, and the list entries the
        inner-product kernels walked, the wedges and triangles of the
        triangle-listing form, and the pruned edges, probed row entries and
        destroyed triangles of the frontier k-truss (device counters)."""
        out = (ctypes.c_int64 * 12)()
        _check(lib().ga_ctx_work_counters(self.handle, out, int(bool(reset))), self)
        return dict(zip(("products", "mask_entries", "launches", "a_entries", "rows", "executed", "executed_dot",
                         "wedges", "triangles", "front_edges", "front_probes", "front_triangles"),
                        (int(x) for x in out)))

    def flush_l2(self):
        _check(lib().ga_ctx_flush_l2(self.handle), self)


def kernel_launches() -> int:
    """Kernel launches issued by the library in this process (host count)."""
    f = lib().ga_kernel_launches
    f.restype = ctypes.c_int64
    return int(f())


def host_register(a: np.ndarray) -> None:
    """Page-lock a numpy array's memory for fast asynchronous copies."""
    _check(lib().ga_host_register(a.ctypes.data_as(_p), ctypes.c_size_t(a.nbytes)))


def host_unregister(a: np.ndarray) -> None:
    _check(lib().ga_host_unregister(a.ctypes.data_as(_p)))


class Csr:
    """Device-resident CSR matrix (the reference's spMtx<T>)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    @classmethod
    def upload(cls, ctx: Context, m: int, n: int, rst, col, val=None, dtype: Optional[int] = None) -> "Csr":
        rst = np.ascontiguousarray(rst, dtype=np.int32)
        col = np.ascontiguousarray(col, dtype=np.int32)
        if val is not None:
            val = np.ascontiguousarray(val)
            if dtype is None:
                dtype = _DT[val.dtype]
            val = np.ascontiguousarray(val, dtype=_NP[dtype])
        elif dtype is None:
            dtype = INT32
        h = _p()
        _check(lib().ga_csr_upload(ctx.handle, _i64(m), _i64(n), _i64(len(col)), _ptr(rst), _ptr(col), _ptr(val),
                                   int(dtype), ctypes.byref(h)), ctx)
        return cls(ctx, h)

    def info(self) -> Tuple[int, int, int, int]:
        m, n, z, d = _i64(), _i64(), _i64(), _int()
        _check(lib().ga_csr_info(self.handle, ctypes.byref(m), ctypes.byref(n), ctypes.byref(z), ctypes.byref(d)))
        return int(m.value), int(n.value), int(z.value), int(d.value)

    @property
    def shape(self):
        m, n, _, _ = self.info()
        return m, n

    @property
    def nnz(self) -> int:
        return self.info()[2]

    @property
    def dtype(self) -> int:
        return self.info()[3]

    def download(self):
        m, n, z, d = self.info()
        rst = np.empty(m + 1, np.int32)
        col = np.empty(z, np.int32)
        val = np.empty(z, _NP[d])
        _check(lib().ga_csr_download(self.ctx.handle, self.handle, _ptr(rst), _ptr(col), _ptr(val)), self.ctx)
        return rst, col, val

    def device_ptrs(self):
        r, c, v = _p(), _p(), _p()
        _check(lib().ga_csr_device_ptrs(self.handle, ctypes.byref(r), ctypes.byref(c), ctypes.byref(v)))
        return int(r.value or 0), int(c.value or 0), int(v.value or 0)

    def set_symmetric(self, symmetric: int = 1) -> None:
        """Declares the matrix symmetric (1: the device check is skipped; a
        false declaration gives wrong results), not symmetric (0), or
        unknown (-1: checked again on the next use)."""
        _check(lib().ga_csr_set_symmetric(self.ctx.handle, self.handle, int(symmetric)), self.ctx)

    def free(self):
        if self.handle:
            lib().ga_csr_free(self.ctx.handle, self.handle)
            self.handle = _p()

    def __del__(self):
        try:
            if self.handle and self.ctx.handle:
                self.free()
        except Exception:
            pass


class Dense:
    """Device-resident row-major dense matrix (the reference's denseMtx<T>)."""

    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    @classmethod
    def create(cls, ctx: Context, m: int, n: int, dtype: int = FP64, values: Optional[np.ndarray] = None):
        h = _p()
        vals = None if values is None else np.ascontiguousarray(values, dtype=_NP[dtype])
        _check(lib().ga_dense_create(ctx.handle, _i64(m), _i64(n), int(dtype), _ptr(vals), ctypes.byref(h)), ctx)
        return cls(ctx, h)

    @classmethod
    def from_csr(cls, A: Csr):
        h = _p()
        _check(lib().ga_dense_from_csr(A.ctx.handle, A.handle, ctypes.byref(h)), A.ctx)
        return cls(A.ctx, h)

    def info(self):
        m, n, d = _i64(), _i64(), _int()
        _check(lib().ga_dense_info(self.handle, ctypes.byref(m), ctypes.byref(n), ctypes.byref(d)))
        return int(m.value), int(n.value), int(d.value)

    def download(self) -> np.ndarray:
        m, n, d = self.info()
        out = np.empty((m, n), _NP[d])
        _check(lib().ga_dense_download(self.ctx.handle, self.handle, _ptr(out)), self.ctx)
        return out

    def free(self):
        if self.handle:
            lib().ga_dense_free(self.ctx.handle, self.handle)
            self.handle = _p()

    def __del__(self):
        try:
            if self.handle and self.ctx.handle:
                self.free()
        except Exception:
            pass


def _algo(a) -> int:
    return ALGOS[a] if isinstance(a, str) else int(a)


def _new(ctx, fn, *args) -> Csr:
    h = _p()
    _check(fn(ctx.handle, *args, ctypes.byref(h)), ctx)
    return Csr(ctx, h)


# ------------------------------------------------------------- operations
def mxm_masked(algo, A: Csr, B: Csr, M: Csr) -> Csr:
    return _new(A.ctx, lib().ga_mxm_masked, _algo(algo), A.handle, B.handle, M.handle)


def mxm_masked_vals(algo, A: Csr, B: Csr, M: Csr, d_cvals: int):
    _check(lib().ga_mxm_masked_vals(A.ctx.handle, _algo(algo), A.handle, B.handle, M.handle, _p(d_cvals)), A.ctx)


def mxm_cmask(A: Csr, B: Csr, M: Csr) -> Csr:
    return _new(A.ctx, lib().ga_mxm_cmask, A.handle, B.handle, M.handle)


def mxm_spd(A: Csr, B: Dense, M: Csr, C: Dense):
    _check(lib().ga_mxm_spd(A.ctx.handle, A.handle, B.handle, M.handle, C.handle), A.ctx)


def add_nointersect(A: Csr, B: Csr) -> Csr:
    return _new(A.ctx, lib().ga_add_nointersect, A.handle, B.handle)


def ewise_mult_masked(A: Dense, B: Dense, M: Csr, C: Dense):
    _check(lib().ga_ewise_mult_masked(A.ctx.handle, A.handle, B.handle, M.handle, C.handle), A.ctx)


def fuse_ewise_mult_add(A: Dense, B: Dense, C: Dense):
    _check(lib().ga_fuse_ewise_mult_add(A.ctx.handle, A.handle, B.handle, C.handle), A.ctx)


def transpose(A: Csr) -> Csr:
    return _new(A.ctx, lib().ga_transpose, A.handle)


def extract_lower(A: Csr) -> Csr:
    return _new(A.ctx, lib().ga_extract_lower, A.handle)


def extract_upper(A: Csr) -> Csr:
    return _new(A.ctx, lib().ga_extract_upper, A.handle)


def symm_from_lower(L: Csr) -> Csr:
    return _new(L.ctx, lib().ga_symm_from_lower, L.handle)


def adjacency(A: Csr) -> Csr:
    return _new(A.ctx, lib().ga_adjacency, A.handle)


def ewise_add(A: Csr, B: Csr, M: Optional[Csr] = None) -> Csr:
    return _new(A.ctx, lib().ga_ewise_add, A.handle, B.handle, M.handle if M is not None else None)


def ewise_mult(A: Csr, B: Csr, M: Optional[Csr] = None) -> Csr:
    return _new(A.ctx, lib().ga_ewise_mult, A.handle, B.handle, M.handle if M is not None else None)


def mult_scalar(A: Csr, alpha: float) -> None:
    """A's values times alpha, in place."""
    _check(lib().ga_mult_scalar(A.ctx.handle, A.handle, ctypes.c_double(alpha)), A.ctx)


def mxv(A: Csr, x: Dense, y: Dense) -> None:
    """y += A x on the device."""
    _check(lib().ga_mxv(A.ctx.handle, A.handle, x.handle, y.handle), A.ctx)


def vxm(A: Csr, x: Dense, y: Dense) -> None:
    """y += x^T A on the device."""
    _check(lib().ga_vxm(A.ctx.handle, A.handle, x.handle, y.handle), A.ctx)


# ------------------------------------------------------------- ingestion
def csr_from_edges(ctx: Context, m: int, n: int, src, dst, val=None, flags: int = 0,
                   dtype: Optional[int] = None) -> Csr:
    """Edge list to a device CSR (rows sorted, duplicates merged onto the
    earliest edge's value); `flags` from EDGES_*."""
    src = np.ascontiguousarray(src, dtype=np.int32)
    dst = np.ascontiguousarray(dst, dtype=np.int32)
    if val is not None:
        val = np.ascontiguousarray(val)
        if dtype is None:
            dtype = _DT[val.dtype]
        val = np.ascontiguousarray(val, dtype=_NP[dtype])
    elif dtype is None:
        dtype = INT32
    h = _p()
    _check(lib().ga_csr_from_edges(ctx.handle, _i64(m), _i64(n), _i64(len(src)), _ptr(src), _ptr(dst), _ptr(val),
                                   int(dtype), int(flags), ctypes.byref(h)), ctx)
    return Csr(ctx, h)


def read_mtx(ctx: Context, path: str, flags: int = 0) -> Tuple[Csr, bytes]:
    """Matrix Market coordinate file parsed on the device, with the
    reference's reader semantics; returns (matrix, 4-byte type code)."""
    h = _p()
    code = ctypes.create_string_buffer(4)
    _check(lib().ga_read_mtx(ctx.handle, os.fsencode(path), int(flags), code, ctypes.byref(h)), ctx)
    return Csr(ctx, h), code.raw


def read_bin(ctx: Context, path: str, flags: int = 0) -> Tuple[Csr, bytes]:
    """Binary CSR file in the reference's layout; returns (matrix, matcode)."""
    h = _p()
    code = ctypes.create_string_buffer(4)
    _check(lib().ga_read_bin(ctx.handle, os.fsencode(path), int(flags), code, ctypes.byref(h)), ctx)
    return Csr(ctx, h), code.raw


def write_bin(A: Csr, path: str, matcode: Optional[bytes] = None) -> None:
    code = None if matcode is None else ctypes.create_string_buffer(bytes(matcode[:4]), 4)
    _check(lib().ga_write_bin(A.ctx.handle, A.handle, code, os.fsencode(path)), A.ctx)


def convert(A: Csr, dtype: int) -> Csr:
    h = _p()
    _check(lib().ga_csr_convert(A.ctx.handle, A.handle, int(dtype), ctypes.byref(h)), A.ctx)
    return Csr(A.ctx, h)


def tc(algo, A: Csr, per_row: bool = True):
    m = A.shape[0]
    total = _i64()
    rows = np.zeros(m, np.int64) if per_row else None
    _check(lib().ga_tc(A.ctx.handle, _algo(algo), A.handle, ctypes.byref(total), _ptr(rows)), A.ctx)
    return int(total.value), rows


def tc_device(algo, A: Csr, total: "Dense"):
    """Device-result triangle count into a 1x1 INT64 Dense (no synchronisation)."""
    ptr = _p()
    _check(lib().ga_dense_device_ptr(total.handle, ctypes.byref(ptr)))
    _check(lib().ga_tc_device(A.ctx.handle, _algo(algo), A.handle, ptr, None), A.ctx)


def tc_lu(algo, A: Csr) -> int:
    total = _i64()
    _check(lib().ga_tc_lu(A.ctx.handle, _algo(algo), A.handle, ctypes.byref(total)), A.ctx)
    return int(total.value)


def tc_vertex(algo, A: Csr) -> np.ndarray:
    out = np.zeros(A.shape[0], np.int32)
    _check(lib().ga_tc_vertex(A.ctx.handle, _algo(algo), A.handle, _ptr(out)), A.ctx)
    return out


def ktruss(algo, A: Csr, k: int) -> Tuple[Csr, int]:
    h = _p()
    it = _int()
    _check(lib().ga_ktruss(A.ctx.handle, _algo(algo), A.handle, int(k), ctypes.byref(h), ctypes.byref(it)), A.ctx)
    return Csr(A.ctx, h), int(it.value)


def ktruss_sweep(algo, A: Csr, kmin: int = 3):
    """k-truss sweep from A: yields (k, C_k, iterations) for k = kmin,
    kmin + 1, ... until C_k is empty (the empty C_k included), each C_k equal
    to ktruss(algo, C_{k-1}, k). The caller frees each C_k."""
    h = _p()
    _check(lib().ga_ktruss_sweep_begin(A.ctx.handle, _algo(algo), A.handle, int(kmin), ctypes.byref(h)), A.ctx)
    try:
        while True:
            c, k, it = _p(), _int(), _int()
            _check(lib().ga_ktruss_sweep_next(h, ctypes.byref(c), ctypes.byref(k), ctypes.byref(it)), A.ctx)
            if not c:
                return
            yield int(k.value), Csr(A.ctx, c), int(it.value)
    finally:
        lib().ga_ktruss_sweep_free(h)


def bc(A: Csr, sources: Sequence[int]) -> np.ndarray:
    src = np.ascontiguousarray(sources, dtype=np.int32)
    out = np.zeros(A.shape[0], np.float64)
    _check(lib().ga_bc(A.ctx.handle, A.handle, _ptr(src), _i64(len(src)), _ptr(out)), A.ctx)
    return out


# ------------------------------------------------------------- generators
def bc_all(A: Csr, block: int) -> np.ndarray:
    """All-source BC in blocks of `block` sources, accumulated on the device
    (betweenness_centrality, include/betweenness_centrality.h:5-123), FP64."""
    out = np.zeros(A.shape[0], dtype=np.float64)
    _check(lib().ga_bc_all(A.ctx.handle, A.handle, _i64(block), _ptr(out)), A.ctx)
    return out


def _take_host(ptr: _p, count: int) -> np.ndarray:
    if count > 0:
        buf = (ctypes.c_int32 * count).from_address(ptr.value)
        out = np.frombuffer(buf, dtype=np.int32).copy()
    else:
        out = np.zeros(0, np.int32)
    lib().ga_host_free(ptr)
    return out


def _gen(fn, *args):
    m, z = _i64(), _i64()
    r, c = _p(), _p()
    _check(fn(*args, ctypes.byref(m), ctypes.byref(z), ctypes.byref(r), ctypes.byref(c)))
    return int(m.value), _take_host(r, int(m.value) + 1), _take_host(c, int(z.value))


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19, seed: int = 1):
    """Seeded R-MAT graph: (m, rst, col), symmetric, sorted, no loops or duplicates."""
    return _gen(lib().ga_gen_rmat, int(scale), int(edge_factor), float(a), float(b), float(c), int(seed))


def gen_rmat_device(ctx: Context, scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19,
                    c: float = 0.19, seed: int = 1) -> Csr:
    """The R-MAT graph of gen_rmat (bit for bit), built on the device."""
    h = _p()
    _check(lib().ga_gen_rmat_device(ctx.handle, int(scale), int(edge_factor), float(a), float(b), float(c),
                                    int(seed), ctypes.byref(h)), ctx)
    return Csr(ctx, h)


def gen_er(n: int, edges: int, seed: int = 1):
    """Seeded Erdos-Renyi G(n, m) graph with `edges` undirected edges."""
    return _gen(lib().ga_gen_er, int(n), int(edges), int(seed))


def gen_knn(n: int, dim: int, k: int = 30, seed: int = 1):
    """Seeded k-NN graph of n Gaussian points in `dim` dimensions, symmetrised."""
    return _gen(lib().ga_gen_knn, int(n), int(dim), int(k), int(seed))


# ------------------------------------------------------------- batched graphs
def _voff_arg(voff) -> np.ndarray:
    return np.ascontiguousarray(voff, dtype=np.int64)


def block_diag(ctx: Context, parts: Sequence[Csr]) -> Tuple[Csr, np.ndarray]:
    """Block-diagonal union of `parts` and its row offsets (count + 1)."""
    handles = (_p * max(1, len(parts)))(*[p.handle for p in parts])
    voff = np.zeros(len(parts) + 1, np.int64)
    h = _p()
    _check(lib().ga_csr_block_diag(ctx.handle, _i64(len(parts)), handles, ctypes.byref(h), _ptr(voff)), ctx)
    return Csr(ctx, h), voff


def gen_knn_batch(ctx: Context, n: Sequence[int], dim: Sequence[int], k: int = 30,
                  seed: int = 1) -> Tuple[Csr, np.ndarray]:
    """Seeded k-NN graphs built on the device, as one block-diagonal union."""
    nn = np.ascontiguousarray(n, dtype=np.int32)
    dd = np.ascontiguousarray(dim, dtype=np.int32)
    if nn.shape != dd.shape:
        raise ValueError("n and dim need one entry per graph")
    voff = np.zeros(len(nn) + 1, np.int64)
    h = _p()
    _check(lib().ga_gen_knn_batch(ctx.handle, _i64(len(nn)), _ptr(nn), _ptr(dd), _int(k), ctypes.c_uint64(seed),
                                  ctypes.byref(h), _ptr(voff)), ctx)
    return Csr(ctx, h), voff


def batch_tc(algo, U: Csr, voff) -> np.ndarray:
    """Per-graph triangle counts of a block-diagonal union."""
    v = _voff_arg(voff)
    out = np.zeros(len(v) - 1, np.int64)
    _check(lib().ga_batch_tc(U.ctx.handle, _algo(algo), U.handle, _i64(len(v) - 1), _ptr(v), _ptr(out)), U.ctx)
    return out


def batch_ktruss(algo, U: Csr, voff, k: int) -> Tuple[Csr, np.ndarray]:
    """Per-graph k-truss of a block-diagonal union: (union of results, iterations per graph)."""
    v = _voff_arg(voff)
    iters = np.zeros(len(v) - 1, np.int32)
    h = _p()
    _check(lib().ga_batch_ktruss(U.ctx.handle, _algo(algo), U.handle, _i64(len(v) - 1), _ptr(v), _int(k),
                                 ctypes.byref(h), _ptr(iters)), U.ctx)
    return Csr(U.ctx, h), iters


def batch_ktruss_k(algo, U: Csr, voff, ks) -> Tuple[Csr, np.ndarray]:
    """Batched k-truss with one k per graph."""
    v = _voff_arg(voff)
    kk = np.ascontiguousarray(ks, dtype=np.int32)
    iters = np.zeros(len(v) - 1, np.int32)
    h = _p()
    _check(lib().ga_batch_ktruss_k(U.ctx.handle, _algo(algo), U.handle, _i64(len(v) - 1), _ptr(v), _ptr(kk),
                                   ctypes.byref(h), _ptr(iters)), U.ctx)
    return Csr(U.ctx, h), iters


def batch_bc(U: Csr, voff, sources_per_graph) -> np.ndarray:
    """Batched BC: one source list (local vertex indices) per graph of the union."""
    v = _voff_arg(voff)
    lists = [np.ascontiguousarray(x, dtype=np.int32) for x in sources_per_graph]
    soff = np.zeros(len(lists) + 1, np.int64)
    soff[1:] = np.cumsum([len(x) for x in lists])
    src = np.concatenate(lists).astype(np.int32) if lists else np.zeros(0, np.int32)
    out = np.zeros(U.shape[0], np.float64)
    _check(lib().ga_batch_bc(U.ctx.handle, U.handle, _i64(len(v) - 1), _ptr(v), _ptr(soff), _ptr(src), _ptr(out)),
           U.ctx)
    return out


def split_blocks(rst: np.ndarray, col: np.ndarray, voff) -> list:
    """Host helper: cut a downloaded block-diagonal CSR into per-graph (m, rst, col)."""
    out = []
    for g in range(len(voff) - 1):
        b, e = int(voff[g]), int(voff[g + 1])
        r = rst[b:e + 1].astype(np.int64)
        out.append((e - b, (r - r[0]).astype(np.int32), (col[r[0]:r[-1]] - b).astype(np.int32)))
    return out


# ------------------------------------------------------------- request server
REQ_TC, REQ_KTRUSS, REQ_BC = 0, 1, 2


class ServerConfig(ctypes.Structure):
    _fields_ = [("workers", _int), ("coalesce", _int), ("tc_algo", _int), ("ktruss_algo", _int),
                ("hbm_budget", _i64), ("coalesce_nnz", _i64), ("coalesce_max_nnz", _i64),
                ("coalesce_max_requests", _i64), ("bc_group_pairs", _i64)]


class ServerResult(ctypes.Structure):
    _fields_ = [("status", _int), ("type", _int), ("graph", _int), ("tc_total", _i64), ("iters", _int),
                ("truss_nnz", _i64), ("truss_rst", ctypes.POINTER(ctypes.c_int32)),
                ("truss_col", ctypes.POINTER(ctypes.c_int32)), ("bc", ctypes.POINTER(ctypes.c_double)),
                ("t_submit", ctypes.c_double), ("t_start", ctypes.c_double), ("t_end", ctypes.c_double),
                ("batch_size", _int), ("worker", _int), ("bytes_bound", _i64), ("error", ctypes.c_char_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, _i64) for n in ("submitted", "completed", "failed", "rejected", "calls", "batched_calls",
                                    "batched_requests", "max_group", "max_in_flight", "budget", "reserved",
                                    "peak_reserved", "queued", "cancelled")]


def request_bytes_bound(req_type: int, m: int, nnz: int, param: int = 0) -> int:
    b = _i64()
    _check(lib().ga_request_bytes_bound(_int(req_type), _i64(m), _i64(nnz), _i64(param), ctypes.byref(b)))
    return int(b.value)


class Server:
    """Request server over device-resident graphs (ga_server_* in the C ABI)."""

    def __init__(self, device: int = 0, workers: int = 4, coalesce: bool = True, tc_algo="msa",
                 ktruss_algo="msa", hbm_budget: int = 0, coalesce_nnz: int = 0, coalesce_max_nnz: int = 0,
                 coalesce_max_requests: int = 0, bc_group_pairs: int = 0):
        cfg = ServerConfig(int(workers), int(bool(coalesce)), _algo(tc_algo), _algo(ktruss_algo), int(hbm_budget),
                           int(coalesce_nnz), int(coalesce_max_nnz), int(coalesce_max_requests),
                           int(bc_group_pairs))
        self.handle = _p()
        self.sizes = []
        _check(lib().ga_server_create(_int(device), ctypes.byref(cfg), ctypes.byref(self.handle)))

    def add_graph(self, m: int, rst, col) -> int:
        rst = np.ascontiguousarray(rst, dtype=np.int32)
        col = np.ascontiguousarray(col, dtype=np.int32)
        gid = _int()
        rc = lib().ga_server_add_graph(self.handle, _i64(m), _ptr(rst), _ptr(col), ctypes.byref(gid))
        if rc != OK:
            raise GaError(rc, lib().ga_status_string(rc).decode())
        self.sizes.append(m)
        return int(gid.value)

    def _added(self, rc: int, gid) -> int:
        if rc != OK:
            raise GaError(rc, lib().ga_status_string(rc).decode())
        m = _i64()
        _check(lib().ga_server_graph_info(self.handle, gid, ctypes.byref(m), None))
        self.sizes.append(int(m.value))
        return int(gid.value)

    def add_graph_device(self, A: Csr) -> int:
        """Copies a symmetric int32 device CSR of the same device into the pool."""
        gid = _int()
        return self._added(lib().ga_server_add_graph_device(self.handle, A.ctx.handle, A.handle, ctypes.byref(gid)),
                           gid)

    def add_graph_file(self, path: str) -> int:
        """Reads a ".mtx" or ".bin" graph file on the device into the pool."""
        gid = _int()
        return self._added(lib().ga_server_add_graph_file(self.handle, os.fsencode(path), ctypes.byref(gid)), gid)

    def submit(self, req_type: int, graph: int, k: int = 0, sources=None, want_edges: bool = False) -> int:
        src = None if sources is None else np.ascontiguousarray(sources, dtype=np.int32)
        rid = _i64()
        _check(lib().ga_server_submit(self.handle, _int(req_type), _int(graph), _int(k), _ptr(src),
                                      _int(0 if src is None else len(src)), _int(int(want_edges)),
                                      ctypes.byref(rid)))
        return int(rid.value)

    def wait(self, rid: int, timeout: float = 0.0, release: bool = True) -> dict:
        r = ServerResult()
        _check(lib().ga_server_wait(self.handle, _i64(rid), ctypes.c_double(timeout), ctypes.byref(r)))
        out = {"status": r.status, "type": r.type, "graph": r.graph, "t_submit": r.t_submit, "t_start": r.t_start,
               "t_end": r.t_end, "batch_size": r.batch_size, "worker": r.worker, "bytes_bound": r.bytes_bound,
               "error": r.error.decode() if r.error else None}
        if r.status == OK:
            if r.type == REQ_TC:
                out["tc"] = int(r.tc_total)
            elif r.type == REQ_KTRUSS:
                out["iters"] = int(r.iters)
                out["nnz"] = int(r.truss_nnz)
                if r.truss_rst:
                    m = self.sizes[r.graph]
                    out["rst"] = np.ctypeslib.as_array(r.truss_rst, (m + 1,)).copy()
                    out["col"] = np.ctypeslib.as_array(r.truss_col, (max(1, r.truss_nnz),))[:r.truss_nnz].copy()
            else:
                out["bc"] = np.ctypeslib.as_array(r.bc, (self.sizes[r.graph],)).copy()
        if release:
            lib().ga_server_release(self.handle, _i64(rid))
        return out

    def cancel(self, rid: int) -> bool:
        """Cancels a request that has not started; False when it already runs
        or ran (it then completes normally)."""
        rc = lib().ga_server_cancel(self.handle, _i64(rid))
        if rc == ERR_UNSUPPORTED:
            return False
        _check(rc)
        return True

    def drain(self, timeout: float = 0.0):
        _check(lib().ga_server_drain(self.handle, ctypes.c_double(timeout)))

    def stats(self) -> dict:
        s = ServerStats()
        _check(lib().ga_server_get_stats(self.handle, ctypes.byref(s)))
        return {n: int(getattr(s, n)) for n, _ in ServerStats._fields_}

    def close(self):
        if self.handle:
            lib().ga_server_destroy(self.handle)
            self.handle = _p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ autotuner
class TuneResult(ctypes.Structure):
    _fields_ = [("algo", _int), ("warp_max_flops", _i64), ("heavy_flops", _i64), ("ctas_per_sm", _int),
                ("dot_chunk", _int), ("hybrid_ratio", _i64), ("ms", ctypes.c_double), ("default_ms", ctypes.c_double),
                ("candidates", _int), ("cached", _int), ("tri_order", _int)]


def autotune(kind: int, A: Csr, B: Optional[Csr] = None, M: Optional[Csr] = None, force: bool = False,
             only=None) -> dict:
    """Tunes (or looks up) the masked-product schedule for A's problem; GA_AUTO
    calls on problems of the same signature use the result. only: restrict to
    one variant ("msa", "mca", "dot")."""
    r = TuneResult()
    algo = -1 if only is None else _algo(only)
    _check(lib().ga_autotune_variant(A.ctx.handle, _int(kind), _int(algo), A.handle, B.handle if B else None,
                                     M.handle if M else None, _int(int(force)), ctypes.byref(r)), A.ctx)
    out = {n: getattr(r, n) for n, _ in TuneResult._fields_}
    out["algo"] = ALGO_NAMES.get(r.algo, r.algo)
    return out


def tune_save(path: str) -> int:
    """Writes the process-wide tuning cache to a file; returns the entries."""
    n = _i64()
    _check(lib().ga_tune_save(os.fsencode(path), ctypes.byref(n)))
    return int(n.value)


def tune_load(path: str) -> int:
    """Adds a saved tuning cache's entries; returns how many."""
    n = _i64()
    _check(lib().ga_tune_load(os.fsencode(path), ctypes.byref(n)))
    return int(n.value)


def tune_clear() -> None:
    _check(lib().ga_tune_clear())


def apply_schedule(ctx: Context, tuned: dict) -> None:
    """Sets a tuning result's schedule as the context's masked-product options."""
    ctx.set_option(OPT_MXM_WARP_FLOPS, tuned["warp_max_flops"])
    ctx.set_option(OPT_MXM_HEAVY_FLOPS, tuned["heavy_flops"])
    ctx.set_option(OPT_MXM_CTAS_PER_SM, tuned["ctas_per_sm"])
    ctx.set_option(OPT_DOT_CHUNK, tuned["dot_chunk"])
    ctx.set_option(OPT_HYBRID_RATIO, tuned.get("hybrid_ratio", 16))
    ctx.set_option(OPT_TRI_ORDER, tuned.get("tri_order", 0))
