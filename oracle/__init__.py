"""ORACLE — test infrastructure only (the CPU reference results the GPU engine is
compared with, and the timed CPU baseline).

Python bindings of oracle/irlba_oracle.cpp, a plain-C++ restatement of CppIrlba's
IRLBA path on column-major arrays. Only tests/, __graft_entry__.smoke() and the
CPU-baseline legs of bench.py use this package; the product never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


class OracleOptions(ctypes.Structure):
    _fields_ = [
        ("invariant_subspace_tolerance", ctypes.c_double),
        ("convergence_tolerance", ctypes.c_double),
        ("singular_value_ratio_tolerance", ctypes.c_double),
        ("extra_work", ctypes.c_int32),
        ("max_iterations", ctypes.c_int32),
        ("exact_for_small_matrix", ctypes.c_int32),
        ("exact_for_large_number", ctypes.c_int32),
        ("cap_number", ctypes.c_int32),
        ("pad0", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("initial", ctypes.POINTER(ctypes.c_double)),
        ("initial_size", ctypes.c_int64),
    ]


class OracleMatrixSpec(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("column_major", ctypes.c_int32),
        ("num_threads", ctypes.c_int32),
        ("center_outer", ctypes.c_int32),
        ("nrow", ctypes.c_int64),
        ("ncol", ctypes.c_int64),
        ("ld", ctypes.c_int64),
        ("dense", ctypes.POINTER(ctypes.c_double)),
        ("values", ctypes.POINTER(ctypes.c_double)),
        ("indices", ctypes.POINTER(ctypes.c_int32)),
        ("pointers", ctypes.POINTER(ctypes.c_int64)),
        ("center", ctypes.POINTER(ctypes.c_double)),
        ("scale", ctypes.POINTER(ctypes.c_double)),
        ("scale_column", ctypes.c_int32),
        ("scale_divide", ctypes.c_int32),
        ("values32", ctypes.POINTER(ctypes.c_float)),
    ]


class OracleError(RuntimeError):
    pass


def load():
    global _lib
    if _lib is not None:
        return _lib
    lib = ctypes.CDLL(_build.build())
    P = ctypes.c_void_p
    pd = ctypes.POINTER(ctypes.c_double)
    i64, i32 = ctypes.c_int64, ctypes.c_int32
    sp = ctypes.POINTER(OracleMatrixSpec)
    op = ctypes.POINTER(OracleOptions)
    lib.oracle_last_error.restype = ctypes.c_char_p
    lib.oracle_set_dense_threads.argtypes = [ctypes.c_int]
    lib.oracle_default_options.argtypes = [op]
    lib.oracle_multiply.argtypes = [sp, pd, pd]
    lib.oracle_adjoint_multiply.argtypes = [sp, pd, pd]
    lib.oracle_realize.argtypes = [sp, pd]
    lib.oracle_sparse_partitions.argtypes = [sp, P, P, P]
    lib.oracle_compute.argtypes = [sp, i64, op, pd, pd, pd, ctypes.POINTER(i64), ctypes.POINTER(i32),
                                   ctypes.POINTER(i32), ctypes.POINTER(i64), i32]
    lib.oracle_pca.argtypes = [sp, i32, i32, i64, op, pd, pd, pd, ctypes.POINTER(i64), ctypes.POINTER(i32),
                               ctypes.POINTER(i32), pd, pd, i32, ctypes.POINTER(i64)]
    lib.oracle_lanczos.argtypes = [sp, pd, pd, pd, i64, i64, ctypes.c_uint64, pd, op]
    lib.oracle_orthogonalize_vector.argtypes = [pd, i64, i64, pd, i64]
    lib.oracle_update_k.restype = i64
    lib.oracle_update_k.argtypes = [i64, i64, i64, i64]
    lib.oracle_requested_ge_half_smaller.restype = i32
    lib.oracle_requested_ge_half_smaller.argtypes = [i64, i64]
    lib.oracle_choose_work.restype = i64
    lib.oracle_choose_work.argtypes = [i64, i32, i64]
    lib.oracle_svd.argtypes = [i64, i64, pd, pd, pd, pd]
    lib.oracle_svd_square.argtypes = [i64, pd, pd, pd, pd]
    lib.oracle_fill_random_normals.argtypes = [pd, i64, ctypes.c_uint64]
    _lib = lib
    return lib


def _pd(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(rc):
    if rc != 0:
        raise OracleError(load().oracle_last_error().decode())


class Spec:
    """Oracle matrix: dense or compressed base plus optional centre/scale."""

    def __init__(self, spec, keep):
        self.spec = spec
        self._keep = keep

    @staticmethod
    def dense(a, center=None, scale=None, scale_column=True, scale_divide=True, center_outer=False):
        a = np.asfortranarray(a, dtype=np.float64)
        s = OracleMatrixSpec()
        s.kind = 0
        s.nrow, s.ncol = a.shape
        s.ld = max(a.shape[0], 1)
        s.dense = _pd(a)
        keep = [a]
        Spec._chain(s, keep, center, scale, scale_column, scale_divide, center_outer)
        return Spec(s, keep)

    @staticmethod
    def sparse(nrow, ncol, x, i, p, column_major, num_threads=1, center=None, scale=None, scale_column=True,
               scale_divide=True, center_outer=False):
        # FP32 values stay FP32 (as a float ValueArray of the reference's
        # ParallelSparseMatrix); products promote them to FP64.
        x = np.ascontiguousarray(x, dtype=np.float32 if np.asarray(x).dtype == np.float32 else np.float64)
        i = np.ascontiguousarray(i, dtype=np.int32)
        p = np.ascontiguousarray(p, dtype=np.int64)
        s = OracleMatrixSpec()
        s.kind = 2
        s.column_major = int(bool(column_major))
        s.num_threads = num_threads
        s.nrow, s.ncol = nrow, ncol
        if x.dtype == np.float32:
            s.values32 = x.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        else:
            s.values = _pd(x)
        s.indices = i.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        s.pointers = p.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))
        keep = [x, i, p]
        Spec._chain(s, keep, center, scale, scale_column, scale_divide, center_outer)
        return Spec(s, keep)

    @staticmethod
    def _chain(s, keep, center, scale, scale_column, scale_divide, center_outer):
        if center is not None:
            c = np.ascontiguousarray(center, dtype=np.float64)
            keep.append(c)
            s.center = _pd(c)
        if scale is not None:
            sc = np.ascontiguousarray(scale, dtype=np.float64)
            keep.append(sc)
            s.scale = _pd(sc)
        s.scale_column = int(bool(scale_column))
        s.scale_divide = int(bool(scale_divide))
        s.center_outer = int(bool(center_outer))

    @property
    def shape(self):
        return self.spec.nrow, self.spec.ncol


def options(**kw):
    o = OracleOptions()
    load().oracle_default_options(ctypes.byref(o))
    keep = []
    for k, v in kw.items():
        if k == "initial":
            if v is not None:
                arr = np.ascontiguousarray(v, dtype=np.float64)
                keep.append(arr)
                o.initial = _pd(arr)
                o.initial_size = arr.shape[0]
        else:
            setattr(o, k, v)
    o._keep = keep
    return o


def multiply(spec, x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty(spec.shape[0])
    _check(load().oracle_multiply(ctypes.byref(spec.spec), _pd(x), _pd(out)))
    return out


def adjoint_multiply(spec, y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    out = np.empty(spec.shape[1])
    _check(load().oracle_adjoint_multiply(ctypes.byref(spec.spec), _pd(y), _pd(out)))
    return out


def realize(spec):
    m, n = spec.shape
    out = np.empty((n, m))
    _check(load().oracle_realize(ctypes.byref(spec.spec), _pd(out)))
    return out.T.copy()


def compute(spec, number, opt=None, max_restarts=-1, dense_threads=1):
    lib = load()
    lib.oracle_set_dense_threads(dense_threads)
    opt = opt or options()
    m, n = spec.shape
    cap = max(min(number, min(m, n)), 0)
    U = np.zeros((max(cap, 1), m))
    V = np.zeros((max(cap, 1), n))
    D = np.zeros(max(cap, 1))
    num = ctypes.c_int64()
    conv = ctypes.c_int32()
    iters = ctypes.c_int32()
    mv = ctypes.c_int64()
    _check(lib.oracle_compute(ctypes.byref(spec.spec), number, ctypes.byref(opt), _pd(U), _pd(V), _pd(D),
                              ctypes.byref(num), ctypes.byref(conv), ctypes.byref(iters), ctypes.byref(mv),
                              max_restarts))
    r = num.value
    return {"U": U[:r].T.copy(), "V": V[:r].T.copy(), "D": D[:r].copy(), "converged": bool(conv.value),
            "iterations": iters.value, "matvecs": mv.value}


def pca(spec, center, scale, number, opt=None, dense_threads=1, max_restarts=-1):
    """pca() (pca.hpp:55-139); max_restarts >= 0 stops after that many restarts
    (a bounded sample for timing)."""
    lib = load()
    lib.oracle_set_dense_threads(dense_threads)
    opt = opt or options()
    m, n = spec.shape
    cap = max(min(number, min(m, n)), 0)
    S = np.zeros((max(cap, 1), m))
    R = np.zeros((max(cap, 1), n))
    var = np.zeros(max(cap, 1))
    c = np.zeros(max(n, 1))
    sc = np.zeros(max(n, 1))
    num = ctypes.c_int64()
    conv = ctypes.c_int32()
    iters = ctypes.c_int32()
    steps = ctypes.c_int64()
    _check(lib.oracle_pca(ctypes.byref(spec.spec), int(bool(center)), int(bool(scale)), number, ctypes.byref(opt),
                          _pd(S), _pd(R), _pd(var), ctypes.byref(num), ctypes.byref(conv), ctypes.byref(iters),
                          _pd(c), _pd(sc), max_restarts, ctypes.byref(steps)))
    r = num.value
    return {"scores": S[:r].T.copy(), "rotation": R[:r].T.copy(), "variances": var[:r].copy(),
            "converged": bool(conv.value), "iterations": iters.value, "center": c[:n].copy(),
            "scale": sc[:n].copy(), "lanczos_steps": steps.value}


def lanczos(spec, W, V, B, start, seed=50, opt=None):
    """run_lanczos_bidiagonalization on copies of W, V, B; returns (W, V, B, F)."""
    m, n = spec.shape
    W = np.asfortranarray(W, dtype=np.float64).copy(order="F")
    V = np.asfortranarray(V, dtype=np.float64).copy(order="F")
    B = np.asfortranarray(B, dtype=np.float64).copy(order="F")
    work = W.shape[1]
    F = np.zeros(n)
    opt = opt or options()
    _check(load().oracle_lanczos(ctypes.byref(spec.spec), _pd(W), _pd(V), _pd(B), work, start, seed, _pd(F),
                                 ctypes.byref(opt)))
    return W, V, B, F


def orthogonalize_vector(Q, v, ncols):
    Q = np.asfortranarray(Q, dtype=np.float64)
    v = np.array(v, dtype=np.float64)
    load().oracle_orthogonalize_vector(_pd(Q), Q.shape[0], Q.shape[1], _pd(v), ncols)
    return v


def update_k(k, requested, n_converged, work):
    return load().oracle_update_k(k, requested, n_converged, work)


def requested_ge_half_smaller(requested, smaller):
    return bool(load().oracle_requested_ge_half_smaller(requested, smaller))


def choose_work(requested, extra_work, smaller):
    return load().oracle_choose_work(requested, extra_work, smaller)


def svd(A):
    A = np.asfortranarray(A, dtype=np.float64)
    m, n = A.shape
    p = min(m, n)
    U = np.zeros((p, m))
    S = np.zeros(p)
    V = np.zeros((p, n))
    load().oracle_svd(m, n, _pd(A), _pd(U), _pd(S), _pd(V))
    return U.T.copy(), S, V.T.copy()


def svd_square(A):
    """The restart loop's SVD of a square B (two-sided Jacobi, as Eigen::JacobiSVD)."""
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    assert A.shape == (n, n)
    U = np.zeros((n, n))
    S = np.zeros(n)
    V = np.zeros((n, n))
    load().oracle_svd_square(n, _pd(A), _pd(U), _pd(S), _pd(V))
    return U.T.copy(), S, V.T.copy()


def scrna_pca_input(genes, cells, density, seed, dtype, cell_major):
    """The seeded single-cell-like PCA input of cppirlba_gb300.datagen, generated
    by the same generator source compiled into the oracle library (so that the
    CPU reference run loads no library of the product)."""
    from cppirlba_gb300 import datagen
    return datagen.scrna_pca_input(genes, cells, density, seed, dtype, cell_major, lib=load())


def random_normals(n, seed):
    out = np.zeros(n)
    load().oracle_fill_random_normals(_pd(out), n, seed)
    return out


def partitions(spec, nt):
    """ParallelSparseMatrix thread partitions (primary, secondary, secondary_nonzero)."""
    s = spec.spec
    s.num_threads = nt
    prim = s.ncol if s.column_major else s.nrow
    pb = np.zeros(nt + 1, dtype=np.int64)
    sb = np.zeros(nt + 1, dtype=np.int64)
    snz = np.zeros((nt + 1) * prim, dtype=np.int64)
    _check(load().oracle_sparse_partitions(ctypes.byref(s), ctypes.c_void_p(pb.ctypes.data),
                                           ctypes.c_void_p(sb.ctypes.data), ctypes.c_void_p(snz.ctypes.data)))
    return pb, sb, snz.reshape(nt + 1, prim)
