"""CPU oracle for the masked-SpGEMM path (test infrastructure only).

ctypes bindings over ``oracle/_build/liboracle.so`` (the plain-C restatement in
``oracle/oracle.c``) and, when it was built on this machine, over
``oracle/_ref/libref.so`` (the unmodified reference compiled by
``oracle/build_ref.sh``). Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline legs of ``bench.py`` import this module; the product never does.

Matrices are plain ``(m, n, rst, col, val)`` tuples of numpy arrays with
int32 ``rst``/``col`` (the reference's ``spMtx`` layout, include/matrix.h:23-33).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import NamedTuple, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libref.so")

_i64 = ctypes.c_int64
_p = ctypes.c_void_p


class Csr(NamedTuple):
    m: int
    n: int
    rst: np.ndarray
    col: np.ndarray
    val: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.rst[self.m])


_SUFFIX = {np.dtype(np.int32): "i32", np.dtype(np.int64): "i64",
           np.dtype(np.float32): "f32", np.dtype(np.float64): "f64"}


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc (OpenMP on)."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("oracle.c", "gen.c")]
    newest = max(os.path.getmtime(f) for f in srcs + [os.path.join(HERE, "oracle.h")])
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        subprocess.check_call(["gcc", "-O2", "-std=c11", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
                               *srcs, "-o", LIB_PATH])
    return LIB_PATH


def build_ref() -> Optional[str]:
    """Compile the unmodified reference into oracle/_ref/libref.so when its
    sources are present on this machine; returns the path or None."""
    script = os.path.join(HERE, "build_ref.sh")
    subprocess.check_call(["bash", script])
    return REF_PATH if os.path.exists(REF_PATH) else None


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.or_tc_sandia.restype = _i64
    return _lib


def reference_dir() -> Optional[str]:
    """The reference source tree oracle/_ref was built from (recorded by
    build_ref.sh), or None where it was not built."""
    try:
        with open(os.path.join(HERE, "_ref", "source_dir")) as f:
            d = f.read().strip()
    except OSError:
        return None
    return d if d and os.path.isdir(d) else None


def ref_available() -> bool:
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        _ref = ctypes.CDLL(REF_PATH)
        _ref.ref_tc_sandia.restype = _i64
    return _ref


def _ptr(a):
    return a.ctypes.data_as(_p) if a is not None else None


def _take(ptr, count, dtype, free):
    """Copy `count` items from a malloc'd pointer into numpy, then free it."""
    dtype = np.dtype(dtype)
    if count > 0:
        buf = (ctypes.c_char * (count * dtype.itemsize)).from_address(ptr.value)
        out = np.frombuffer(bytes(buf), dtype=dtype).copy()
    else:
        out = np.zeros(0, dtype=dtype)
    free(ptr)
    return out


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def set_num_threads(n: int) -> None:
    lib().or_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().or_num_threads())


# ---------------------------------------------------------------- restatement
def mxm_masked(A: Csr, B: Csr, M: Csr) -> np.ndarray:
    """Values of C<M> = A*B on M's pattern (matrix_la.h:715-749)."""
    dt = np.dtype(A.val.dtype)
    s = _SUFFIX[dt]
    cv = np.zeros(M.nnz, dtype=dt)
    fn = getattr(lib(), f"or_mxm_masked_{s}")
    fn(_i64(A.m), _i64(B.n), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
       _ptr(_c(B.rst, np.int32)), _ptr(_c(B.col, np.int32)), _ptr(_c(B.val, dt)),
       _ptr(_c(M.rst, np.int32)), _ptr(_c(M.col, np.int32)), _ptr(cv))
    return cv


def _new_csr(fn, m, n, dt, *args):
    cr, cc, cv = _p(), _p(), _p()
    cnz = _i64()
    fn(*args, ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv), ctypes.byref(cnz))
    free = lib().or_free
    rst = _take(cr, m + 1, np.int32, free)
    z = int(rst[m]) if m >= 0 else 0
    return Csr(m, n, rst, _take(cc, z, np.int32, free), _take(cv, z, dt, free))


def mxm_cmask(A: Csr, B: Csr, M: Csr) -> Csr:
    """C<!M> = A*B with a new, sorted pattern (matrix_la.h:800-891)."""
    dt = np.dtype(A.val.dtype)
    fn = getattr(lib(), f"or_mxm_cmask_{_SUFFIX[dt]}")
    return _new_csr(fn, A.m, B.n, dt, _i64(A.m), _i64(B.n),
                    _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
                    _ptr(_c(B.rst, np.int32)), _ptr(_c(B.col, np.int32)), _ptr(_c(B.val, dt)),
                    _ptr(_c(M.rst, np.int32)), _ptr(_c(M.col, np.int32)))


def mxm_spd(A: Csr, Bd: np.ndarray, M: Csr) -> np.ndarray:
    """Dense C<M> = A * Bd (matrix_la.h:241-270)."""
    dt = np.dtype(A.val.dtype)
    Bd = _c(Bd, dt)
    n = Bd.shape[1]
    C = np.zeros((A.m, n), dtype=dt)
    getattr(lib(), f"or_mxm_spd_{_SUFFIX[dt]}")(
        _i64(A.m), _i64(n), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
        _ptr(Bd), _ptr(_c(M.rst, np.int32)), _ptr(_c(M.col, np.int32)), _ptr(C))
    return C


def add_nointersect(A: Csr, B: Csr) -> Csr:
    dt = np.dtype(A.val.dtype)
    fn = getattr(lib(), f"or_add_nointersect_{_SUFFIX[dt]}")
    return _new_csr(fn, A.m, A.n, dt, _i64(A.m),
                    _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
                    _ptr(_c(B.rst, np.int32)), _ptr(_c(B.col, np.int32)), _ptr(_c(B.val, dt)))


def ewise_mult_masked(Ad: np.ndarray, Bd: np.ndarray, M: Csr) -> np.ndarray:
    dt = Ad.dtype
    C = np.zeros_like(Ad)
    getattr(lib(), f"or_ewise_mult_masked_{_SUFFIX[np.dtype(dt)]}")(
        _i64(Ad.shape[0]), _i64(Ad.shape[1]), _ptr(_c(Ad, dt)), _ptr(_c(Bd, dt)),
        _ptr(_c(M.rst, np.int32)), _ptr(_c(M.col, np.int32)), _ptr(C))
    return C


def fuse_ewise_mult_add(Ad: np.ndarray, Bd: np.ndarray, Cd: np.ndarray) -> np.ndarray:
    C = np.array(Cd, copy=True)
    getattr(lib(), f"or_fuse_ewise_mult_add_{_SUFFIX[np.dtype(C.dtype)]}")(
        _i64(C.size), _ptr(_c(Ad, C.dtype)), _ptr(_c(Bd, C.dtype)), _ptr(C))
    return C


def _maybe(X: Optional[Csr], field: str):
    return _ptr(_c(getattr(X, field), np.int32)) if X is not None else None


def ewise_add(A: Csr, B: Csr, M: Optional[Csr] = None) -> Csr:
    """eWiseAdd (matrix_la.h:375-435), or its masked form (272-335) when M is given."""
    dt = np.dtype(A.val.dtype)
    fn = getattr(lib(), f"or_ewise_add_{_SUFFIX[dt]}")
    return _new_csr(fn, A.m, A.n, dt, _i64(A.m),
                    _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
                    _ptr(_c(B.rst, np.int32)), _ptr(_c(B.col, np.int32)), _ptr(_c(B.val, dt)),
                    _maybe(M, "rst"), _maybe(M, "col"))


def ewise_mult(A: Csr, B: Csr, M: Optional[Csr] = None) -> Csr:
    """eWiseMult on sparse operands (matrix_la.h:438-533)."""
    dt = np.dtype(A.val.dtype)
    fn = getattr(lib(), f"or_ewise_mult_{_SUFFIX[dt]}")
    return _new_csr(fn, A.m, A.n, dt, _i64(A.m),
                    _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
                    _ptr(_c(B.rst, np.int32)), _ptr(_c(B.col, np.int32)), _ptr(_c(B.val, dt)),
                    _maybe(M, "rst"), _maybe(M, "col"))


def mult_scalar(A: Csr, alpha: float) -> Csr:
    """multScalar (matrix_la.h:535-541) on a copy of A."""
    dt = np.dtype(A.val.dtype)
    v = np.array(A.val[: A.nnz], dtype=dt, copy=True)
    getattr(lib(), f"or_mult_scalar_{_SUFFIX[dt]}")(_i64(len(v)), _ptr(v), ctypes.c_double(alpha))
    return Csr(A.m, A.n, A.rst.copy(), A.col.copy(), v)


def mxv(A: Csr, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """y + A x in row order (MxV, matrix_la.h:1279-1284)."""
    dt = np.dtype(A.val.dtype)
    out = np.array(y, dtype=dt, copy=True)
    getattr(lib(), f"or_mxv_{_SUFFIX[dt]}")(_i64(A.m), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)),
                                            _ptr(_c(A.val, dt)), _ptr(_c(x, dt)), _ptr(out))
    return out


def vxm(A: Csr, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """y + x^T A with rows taken in ascending order (VxM, matrix_la.h:1286-1291)."""
    dt = np.dtype(A.val.dtype)
    out = np.array(y, dtype=dt, copy=True)
    getattr(lib(), f"or_vxm_{_SUFFIX[dt]}")(_i64(A.m), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)),
                                            _ptr(_c(A.val, dt)), _ptr(_c(x, dt)), _ptr(out))
    return out


def transpose(A: Csr) -> Csr:
    dt = np.dtype(A.val.dtype)
    cr, cc, cv = _p(), _p(), _p()
    getattr(lib(), f"or_transpose_{_SUFFIX[dt]}")(
        _i64(A.m), _i64(A.n), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
        ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv))
    free = lib().or_free
    rst = _take(cr, A.n + 1, np.int32, free)
    z = A.nnz
    return Csr(A.n, A.m, rst, _take(cc, z, np.int32, free), _take(cv, z, dt, free))


def _tri(name, A: Csr) -> Csr:
    dt = np.dtype(A.val.dtype)
    fn = getattr(lib(), f"or_{name}_{_SUFFIX[dt]}")
    return _new_csr(fn, A.m, A.n, dt, _i64(A.m), _ptr(_c(A.rst, np.int32)),
                    _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)))


def extract_lower(A: Csr) -> Csr:
    return _tri("extract_lower", A)


def extract_upper(A: Csr) -> Csr:
    return _tri("extract_upper", A)


def symm_from_lower(L: Csr) -> Csr:
    return _tri("symm_from_lower", L)


def gen_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             seed: int = 1):
    """Seeded R-MAT graph (oracle/gen.c): (m, rst, col), the same graph as
    the product's generator gives for the same arguments."""
    m, z = _i64(), _i64()
    cr, cc = _p(), _p()
    rc = lib().or_gen_rmat(int(scale), int(edge_factor), ctypes.c_double(a), ctypes.c_double(b),
                           ctypes.c_double(c), ctypes.c_uint64(seed), ctypes.byref(m), ctypes.byref(z),
                           ctypes.byref(cr), ctypes.byref(cc))
    if rc != 0:
        raise RuntimeError(f"or_gen_rmat failed ({rc})")
    free = lib().or_free
    rst = _take(cr, m.value + 1, np.int32, free)
    return int(m.value), rst, _take(cc, z.value, np.int32, free)


def tc_sandia(A: Csr):
    """(total, per-row counts) of main.cpp:65-86."""
    rows = np.zeros(A.m, dtype=np.int64)
    total = lib().or_tc_sandia(_i64(A.m), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(rows))
    return int(total), rows


def ktruss(A: Csr, k: int, with_products: bool = False):
    """(pattern CSR, iterations) of main.cpp:90-146; with_products adds the
    Gustavson product count of all its support products."""
    cr, cc, cv = _p(), _p(), _p()
    cnz = _i64()
    it = ctypes.c_int()
    prod = _i64()
    val = _c(A.val, np.int32) if A.val is not None else None
    lib().or_ktruss_ex(_i64(A.m), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(val), int(k),
                       ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv), ctypes.byref(cnz), ctypes.byref(it),
                       ctypes.byref(prod))
    free = lib().or_free
    rst = _take(cr, A.m + 1, np.int32, free)
    z = int(cnz.value)
    C = Csr(A.m, A.n, rst, _take(cc, z, np.int32, free), _take(cv, z, np.int32, free))
    if with_products:
        return C, int(it.value), int(prod.value)
    return C, int(it.value)


def bc_batch(A: Csr, sources) -> np.ndarray:
    """FP64 batched BC over an explicit source list (betweenness_centrality.h:125-237)."""
    src = _c(sources, np.int32)
    bc = np.zeros(A.m, dtype=np.float64)
    val = _c(A.val, np.int32) if A.val is not None else None
    lib().or_bc_batch(_i64(A.m), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(val),
                      _i64(len(src)), _ptr(src), _ptr(bc))
    return bc


def bc_all(A: Csr, block: int) -> np.ndarray:
    """FP64 all-source BC in blocks of `block` sources (betweenness_centrality.h:5-123)."""
    bc = np.zeros(A.m, dtype=np.float64)
    val = _c(A.val, np.int32) if A.val is not None else None
    rc = lib().or_bc_all(_i64(A.m), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(val),
                         _i64(block), _ptr(bc))
    if rc != 0:
        raise ValueError("block must be at least 1")
    return bc


# ----------------------------------------------------- unmodified reference
def _ref_new(fn, dt, *args):
    cm, cn, cnz = _i64(), _i64(), _i64()
    cr, cc, cv = _p(), _p(), _p()
    rc = fn(*args, ctypes.byref(cm), ctypes.byref(cn), ctypes.byref(cnz),
            ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv))
    if rc != 0:
        raise RuntimeError("reference call failed")
    free = ref().ref_free
    m = int(cm.value)
    rst = _take(cr, m + 1, np.int32, free)
    z = int(cnz.value)
    return Csr(m, int(cn.value), rst, _take(cc, z, np.int32, free), _take(cv, z, dt, free))


def _ref_args(X: Csr, dt):
    return (_i64(X.m), _i64(X.n), _i64(X.nnz), _ptr(_c(X.rst, np.int32)), _ptr(_c(X.col, np.int32)),
            _ptr(_c(X.val, dt)))


def ref_read_mtx(path: str, symmetrise: bool = True) -> Csr:
    m, n, z = _i64(), _i64(), _i64()
    cr, cc, cv = _p(), _p(), _p()
    rc = ref().ref_read_mtx(path.encode(), int(symmetrise), ctypes.byref(m), ctypes.byref(n),
                            ctypes.byref(z), ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv))
    if rc != 0:
        raise RuntimeError(f"reference could not read {path}")
    free = ref().ref_free
    rst = _take(cr, m.value + 1, np.int32, free)
    return Csr(int(m.value), int(n.value), rst, _take(cc, z.value, np.int32, free),
               _take(cv, z.value, np.int32, free))


def read_mtx_cli(path: str, symmetrise: bool = True) -> Csr:
    """The C port of the reference CLI's Matrix Market reading and graph
    preparation (or_read_mtx_cli); values 1."""
    m, z = _i64(), _i64()
    cr, cc = _p(), _p()
    if lib().or_read_mtx_cli(path.encode(), int(symmetrise), ctypes.byref(m), ctypes.byref(z), ctypes.byref(cr),
                             ctypes.byref(cc)) != 0:
        raise RuntimeError(f"cannot read {path}")
    free = lib().or_free
    rst = _take(cr, m.value + 1, np.int32, free)
    return Csr(int(m.value), int(m.value), rst, _take(cc, z.value, np.int32, free), np.ones(z.value, np.int32))


def ref_read_raw(path: str, fmt: str):
    """The reference's reader on `path` (format "mtx", "bin", ...), before
    build_adjacency_matrix: (Csr with float64 values, matcode bytes)."""
    m, n, z = _i64(), _i64(), _i64()
    cr, cc, cv = _p(), _p(), _p()
    code = ctypes.create_string_buffer(4)
    rc = ref().ref_read_raw(path.encode(), fmt.encode(), ctypes.byref(m), ctypes.byref(n), ctypes.byref(z),
                            ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv), code)
    if rc != 0:
        raise RuntimeError(f"reference could not read {path}")
    free = ref().ref_free
    rst = _take(cr, m.value + 1, np.int32, free)
    return (Csr(int(m.value), int(n.value), rst, _take(cc, z.value, np.int32, free),
                _take(cv, z.value, np.float64, free)), code.raw)


def ref_read_cli(path: str, fmt: str, symmetrise: bool) -> Csr:
    """The reference CLI's graph preparation (read, adjacency, and the
    lower-triangle symmetrisation when `symmetrise`)."""
    m, n, z = _i64(), _i64(), _i64()
    cr, cc, cv = _p(), _p(), _p()
    rc = ref().ref_read_cli(path.encode(), fmt.encode(), int(symmetrise), ctypes.byref(m), ctypes.byref(n),
                            ctypes.byref(z), ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv))
    if rc != 0:
        raise RuntimeError(f"reference could not read {path}")
    free = ref().ref_free
    rst = _take(cr, m.value + 1, np.int32, free)
    return Csr(int(m.value), int(n.value), rst, _take(cc, z.value, np.int32, free),
               _take(cv, z.value, np.int32, free))


def ref_tobinary(path: str, fmt: str, out_path: str) -> None:
    """The reference CLI's "tobinary" action on `path`, written to `out_path`."""
    if ref().ref_tobinary(path.encode(), fmt.encode(), out_path.encode()) != 0:
        raise RuntimeError(f"reference could not convert {path}")


def ref_ewise_add(A: Csr, B: Csr, M: Optional[Csr] = None) -> Csr:
    """The reference's eWiseAdd (masked when M is given); int32 or float64."""
    dt = np.dtype(A.val.dtype)
    fn = ref().ref_ewise_add_i32 if dt == np.int32 else ref().ref_ewise_add_f64
    Mx = M if M is not None else A
    return _ref_new(fn, dt, ctypes.c_int(M is not None), _i64(A.m), _i64(A.n), _i64(A.nnz),
                    _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, dt)),
                    _i64(B.nnz), _ptr(_c(B.rst, np.int32)), _ptr(_c(B.col, np.int32)), _ptr(_c(B.val, dt)),
                    _i64(Mx.nnz), _ptr(_c(Mx.rst, np.int32)), _ptr(_c(Mx.col, np.int32)))


def ref_vxm(A: Csr, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    dt = np.dtype(A.val.dtype)
    out = np.array(y, dtype=dt, copy=True)
    xx = np.array(x, dtype=dt, copy=True)
    fn = ref().ref_vxm_i32 if dt == np.int32 else ref().ref_vxm_f64
    if fn(*_ref_args(A, dt), _ptr(xx), _ptr(out)) != 0:
        raise RuntimeError("reference call failed")
    return out


def ref_mxm(algo: int, A: Csr, B: Csr, M: Csr) -> Csr:
    """Reference C<M> = A*B; algo 0 msa, 1 mca, 2 heap (zero-filled C), 3 naive."""
    dt = np.dtype(A.val.dtype)
    fn = ref().ref_mxm_i32 if dt == np.int32 else ref().ref_mxm_f64
    return _ref_new(fn, dt, ctypes.c_int(algo), *_ref_args(A, dt), *_ref_args(B, dt), *_ref_args(M, dt))


def ref_cmask(A: Csr, B: Csr, M: Csr) -> Csr:
    dt = np.dtype(A.val.dtype)
    fn = ref().ref_cmask_i32 if dt == np.int32 else ref().ref_cmask_f64
    return _ref_new(fn, dt, *_ref_args(A, dt), *_ref_args(B, dt), *_ref_args(M, dt))


def ref_tc(A: Csr, algo: int = 0):
    total = ref().ref_tc_sandia(ctypes.c_int(algo), _i64(A.m), _i64(A.nnz), _ptr(_c(A.rst, np.int32)),
                                _ptr(_c(A.col, np.int32)))
    rows = np.zeros(A.m, dtype=np.int64)
    ref().ref_tc_rows(_i64(A.m), _i64(A.nnz), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)),
                      _ptr(rows))
    return int(total), rows


def ref_ktruss(A: Csr, k: int, algo: int = 0):
    cnz = _i64()
    cr, cc, cv = _p(), _p(), _p()
    it = ctypes.c_int()
    rc = ref().ref_ktruss(ctypes.c_int(algo), _i64(A.m), _i64(A.nnz), _ptr(_c(A.rst, np.int32)),
                          _ptr(_c(A.col, np.int32)), _ptr(_c(A.val, np.int32)), ctypes.c_int(k),
                          ctypes.byref(cnz), ctypes.byref(cr), ctypes.byref(cc), ctypes.byref(cv),
                          ctypes.byref(it))
    if rc != 0:
        raise RuntimeError("reference k_truss failed")
    free = ref().ref_free
    rst = _take(cr, A.m + 1, np.int32, free)
    z = int(cnz.value)
    return Csr(A.m, A.n, rst, _take(cc, z, np.int32, free), _take(cv, z, np.int32, free)), int(it.value)


def ref_bc_f32(A: Csr, batch: int) -> np.ndarray:
    bc = np.zeros(A.m, dtype=np.float32)
    ref().ref_bc_batch_f32(_i64(A.m), _i64(A.nnz), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)),
                           _i64(batch), _ptr(bc))
    return bc


def ref_bc_all_f32(A: Csr, block: int) -> np.ndarray:
    """The reference's betweenness_centrality as shipped (FP32, all sources)."""
    bc = np.zeros(A.m, dtype=np.float32)
    ref().ref_bc_all_f32(_i64(A.m), _i64(A.nnz), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)),
                         _i64(block), _ptr(bc))
    return bc


def ref_bc_f64(A: Csr, sources) -> np.ndarray:
    src = _c(sources, np.int32)
    bc = np.zeros(A.m, dtype=np.float64)
    ref().ref_bc_batch_f64(_i64(A.m), _i64(A.nnz), _ptr(_c(A.rst, np.int32)), _ptr(_c(A.col, np.int32)),
                           _ptr(_c(A.val, np.int32)), _i64(len(src)), _ptr(src), _ptr(bc))
    return bc
