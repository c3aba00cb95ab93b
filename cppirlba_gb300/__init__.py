"""GB300 (sm_103a) IRLBA engine: Python mirror of CppIrlba's interface.

The names follow CppIrlba (irlba::Options, irlba::compute, irlba::compute_simple,
irlba::pca, irlba::ParallelSparseMatrix, irlba::SimpleMatrix,
irlba::CenteredMatrix, irlba::ScaledMatrix) and every call goes through the C
ABI declared in include/irlba_gb300.h. There is no CPU fallback: if the CUDA
library is missing or no GPU is visible, the calls raise.
"""
import ctypes
import os
import threading
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libirlba_gb300.so")

FORM_FP64 = 0
FORM_FP32_FP64STEPS = 1
VALUE_F32 = 0
VALUE_F64 = 1

OK = 0
ERROR_INVALID_ARGUMENT = 1
ERROR_CUDA = 2
ERROR_NUMERICAL = 3
ERROR_UNSUPPORTED = 4


class IrlbaError(RuntimeError):
    """An engine call failed; `status` is the irlba_gb300_status code."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class _Options(ctypes.Structure):
    _fields_ = [
        ("invariant_subspace_tolerance", ctypes.c_double),
        ("convergence_tolerance", ctypes.c_double),
        ("singular_value_ratio_tolerance", ctypes.c_double),
        ("extra_work", ctypes.c_int32),
        ("max_iterations", ctypes.c_int32),
        ("exact_for_small_matrix", ctypes.c_int32),
        ("exact_for_large_number", ctypes.c_int32),
        ("cap_number", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("initial", ctypes.POINTER(ctypes.c_double)),
        ("initial_size", ctypes.c_int64),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("matvecs", ctypes.c_int64),
        ("lanczos_steps", ctypes.c_int64),
        ("restarts", ctypes.c_int64),
        ("careful_restarts", ctypes.c_int64),
        ("seconds_total", ctypes.c_double),
        ("device_ms", ctypes.c_double),
        ("kernel_launches", ctypes.c_int64),
        ("svd_sweeps", ctypes.c_int64),
    ]


class BatchInfo(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int32),
        ("converged", ctypes.c_int32),
        ("iterations", ctypes.c_int32),
        ("group_mul", ctypes.c_int32),
        ("group_adj", ctypes.c_int32),
        ("prefetch_mul", ctypes.c_int32),
        ("prefetch_adj", ctypes.c_int32),
        ("error", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("lanczos_steps", ctypes.c_int64),
        ("svd_sweeps", ctypes.c_int64),
        ("ms", ctypes.c_double),
    ]


class BatchStats(ctypes.Structure):
    _fields_ = [
        ("device_ms", ctypes.c_double),
        ("tune_ms", ctypes.c_double),
        ("single_ms", ctypes.c_double),
        ("kernel_launches", ctypes.c_int64),
        ("graph_captured", ctypes.c_int32),
        ("single", ctypes.c_int32),
        ("ctas", ctypes.c_int32),
        ("team", ctypes.c_int32),
        ("joint", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("nnz", ctypes.c_int64),
        ("lanczos_steps", ctypes.c_int64),
    ]


BATCH_OK, BATCH_SINGLE, BATCH_FAILED = 0, 1, 2

_lib = None


def library_path():
    return _LIB_PATH


def load_library():
    """Load the engine (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        from . import build as _build
        _build.build()
    lib = ctypes.CDLL(_LIB_PATH)
    P = ctypes.c_void_p
    i64, i32, dbl = ctypes.c_int64, ctypes.c_int32, ctypes.c_double
    pd = ctypes.POINTER(ctypes.c_double)
    sig = {
        "irlba_gb300_default_options": (None, [ctypes.POINTER(_Options)]),
        "irlba_gb300_last_error": (ctypes.c_char_p, []),
        "irlba_gb300_device_count": (ctypes.c_int, []),
        "irlba_gb300_matrix_create_sparse": (i32, [i64, i64, P, i32, P, P, i32, i32, ctypes.POINTER(P)]),
        "irlba_gb300_matrix_create_dense": (i32, [i64, i64, P, i32, i64, i32, i32, ctypes.POINTER(P)]),
        "irlba_gb300_matrix_create_device_operator": (i32, [i64, i64, P, P, i32, ctypes.POINTER(P)]),
        "irlba_gb300_matrix_create_host_operator": (i32, [i64, i64, P, P, i32, ctypes.POINTER(P)]),
        "irlba_gb300_matrix_center": (i32, [P, pd, ctypes.POINTER(P)]),
        "irlba_gb300_matrix_scale": (i32, [P, pd, i32, i32, ctypes.POINTER(P)]),
        "irlba_gb300_matrix_destroy": (i32, [P]),
        "irlba_gb300_matrix_dims": (i32, [P, ctypes.POINTER(i64), ctypes.POINTER(i64)]),
        "irlba_gb300_multiply": (i32, [P, pd, pd]),
        "irlba_gb300_adjoint_multiply": (i32, [P, pd, pd]),
        "irlba_gb300_realize": (i32, [P, pd]),
        "irlba_gb300_compute": (i32, [P, i64, ctypes.POINTER(_Options), pd, pd, pd, ctypes.POINTER(i64),
                                      ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(Stats)]),
        "irlba_gb300_compute_device": (i32, [P, i64, ctypes.POINTER(_Options), P, P, P, ctypes.POINTER(i64),
                                             ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(Stats), P]),
        "irlba_gb300_pca": (i32, [P, i32, i32, i64, ctypes.POINTER(_Options), pd, pd, pd, ctypes.POINTER(i64),
                                  ctypes.POINTER(i32), ctypes.POINTER(i32), pd, pd, ctypes.POINTER(Stats)]),
        "irlba_gb300_pca_device": (i32, [P, i32, i32, i64, ctypes.POINTER(_Options), P, P, P, ctypes.POINTER(i64),
                                         ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(Stats), P]),
        "irlba_gb300_orthogonalize_vector_device": (i32, [P, i64, i64, i64, P, P]),
        "irlba_gb300_spmv_device": (i32, [P, i32, P, P, P]),
        "irlba_gb300_matrix_set_vector": (i32, [P, pd]),
        "irlba_gb300_update_k_device": (i32, [P, i64, P]),
        "irlba_gb300_matrix_layout": (i32, [P, ctypes.POINTER(i64), ctypes.POINTER(i32), ctypes.POINTER(i32),
                                            ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32)]),
        "irlba_gb300_set_profiling": (None, [i32]),
        "irlba_gb300_set_device_ingest": (None, [i32]),
        "irlba_gb300_set_spmv_shape": (None, [i32]),
        "irlba_gb300_set_rotation_engine": (None, [i32]),
        "irlba_gb300_set_value_coding": (None, [i32]),
        "irlba_gb300_rotate_device": (i32, [i32, P, i64, i64, i32, P, i32, i32, P, i64, P, P, i32, P]),
        "irlba_gb300_set_staging": (None, [i64, i64]),
        "irlba_gb300_last_profile": (None, [pd, ctypes.POINTER(i64)]),
        "irlba_gb300_launch_count": (i64, []),
        "irlba_gb300_transfer_bytes": (None, [ctypes.POINTER(i64), ctypes.POINTER(i64)]),
        "irlba_gb300_batch_create": (i32, [i32, P, P, P, i32, P, P, i32, ctypes.POINTER(P)]),
        "irlba_gb300_batch_destroy": (i32, [P]),
        "irlba_gb300_batch_tune": (i32, [P, i32, P]),
        "irlba_gb300_batch_set_team": (i32, [P, i32, i32]),
        "irlba_gb300_batch_groups": (i32, [P, P, P]),
        "irlba_gb300_batch_set_groups": (i32, [P, P, P]),
        "irlba_gb300_batch_pca": (i32, [P, i32, i32, i64, ctypes.POINTER(_Options), ctypes.POINTER(BatchStats), P]),
        "irlba_gb300_batch_result": (i32, [P, i32, pd, pd, pd, pd, pd, ctypes.POINTER(BatchInfo)]),
        "irlba_gb300_batch_result_device": (i32, [P, i32, ctypes.POINTER(P), ctypes.POINTER(P), ctypes.POINTER(P)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


# The Python exception raised inside a user-defined product (OperatorMatrix,
# DeviceOperatorMatrix) on this thread, re-raised as the cause of the failing call.
_callback_state = threading.local()


def _check(status):
    if status != OK:
        msg = load_library().irlba_gb300_last_error().decode()
        cause = getattr(_callback_state, "error", None)
        _callback_state.error = None
        if cause is not None:
            raise IrlbaError(status, msg) from cause
        raise IrlbaError(status, msg)


def _is_scipy_sparse(a):
    try:
        import scipy.sparse as sp
    except ImportError:
        return False
    return sp.issparse(a)


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _vptr(a):
    return ctypes.c_void_p(a.ctypes.data)


@dataclass
class Options:
    """irlba::Options (Options.hpp:19-83): same field names and defaults."""

    invariant_subspace_tolerance: float = -1.0
    convergence_tolerance: float = 1e-5
    singular_value_ratio_tolerance: float = -1.0
    extra_work: int = 7
    max_iterations: int = 1000
    exact_for_small_matrix: bool = True
    exact_for_large_number: bool = True
    cap_number: bool = False
    seed: int = 5489
    initial: Optional[np.ndarray] = None

    def _to_c(self, keep):
        o = _Options()
        o.invariant_subspace_tolerance = self.invariant_subspace_tolerance
        o.convergence_tolerance = self.convergence_tolerance
        o.singular_value_ratio_tolerance = self.singular_value_ratio_tolerance
        o.extra_work = self.extra_work
        o.max_iterations = self.max_iterations
        o.exact_for_small_matrix = int(self.exact_for_small_matrix)
        o.exact_for_large_number = int(self.exact_for_large_number)
        o.cap_number = int(self.cap_number)
        o.reserved0 = 0
        o.seed = self.seed
        if self.initial is not None:
            init = np.ascontiguousarray(self.initial, dtype=np.float64)
            keep.append(init)
            o.initial = _dptr(init)
            o.initial_size = init.shape[0]
        else:
            o.initial = None
            o.initial_size = 0
        return o


@dataclass
class Results:
    """irlba::Results (compute.hpp:357-388). U and V are column-major
    (Fortran-ordered) like the reference's Eigen matrices."""

    U: np.ndarray
    V: np.ndarray
    D: np.ndarray
    iterations: int
    converged: bool
    stats: Optional[dict] = None


@dataclass
class PcaResults:
    """irlba::PcaResults (pca.hpp:146-179). scores and rotation are
    column-major (Fortran-ordered) like the reference's Eigen matrices."""

    scores: np.ndarray
    rotation: np.ndarray
    variances: np.ndarray
    iterations: int
    converged: bool
    center: Optional[np.ndarray] = None
    scale: Optional[np.ndarray] = None
    stats: Optional[dict] = None


def _stats_dict(st):
    return {f: getattr(st, f) for f, _ in Stats._fields_}


class Matrix:
    """irlba::Matrix (Matrix/interface.hpp:141-223) backed by a device handle."""

    def __init__(self, handle, nrow, ncol, form, keep=()):
        self._h = ctypes.c_void_p(handle)
        self._nrow = nrow
        self._ncol = ncol
        self.form = form
        self._keep = list(keep)

    def rows(self):
        return self._nrow

    def cols(self):
        return self._ncol

    @property
    def handle(self):
        return self._h

    def multiply(self, right, output=None):
        """Workspace::multiply (interface.hpp:49): output = A @ right."""
        right = np.ascontiguousarray(right, dtype=np.float64)
        if right.shape != (self._ncol,):
            raise ValueError("right must have length cols()")
        out = np.empty(self._nrow) if output is None else output
        _check(load_library().irlba_gb300_multiply(self._h, _dptr(right), _dptr(out)))
        return out

    def adjoint_multiply(self, right, output=None):
        """AdjointWorkspace::multiply (interface.hpp:87): output = A.T @ right."""
        right = np.ascontiguousarray(right, dtype=np.float64)
        if right.shape != (self._nrow,):
            raise ValueError("right must have length rows()")
        out = np.empty(self._ncol) if output is None else output
        _check(load_library().irlba_gb300_adjoint_multiply(self._h, _dptr(right), _dptr(out)))
        return out

    def realize(self):
        """RealizeWorkspace::realize_copy (interface.hpp:125-130)."""
        out = np.empty((self._ncol, self._nrow))  # column-major buffer
        _check(load_library().irlba_gb300_realize(self._h, _dptr(out)))
        return out.T.copy()

    def close(self):
        if self._h is not None and self._h.value:
            load_library().irlba_gb300_matrix_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ParallelSparseMatrix(Matrix):
    """irlba::ParallelSparseMatrix(nrow, ncol, x, i, p, column_major, num_threads)
    (Matrix/sparse.hpp:469). num_threads is accepted for interface parity; the
    device decides its own work split."""

    def __init__(self, nrow, ncol, x, i, p, column_major, num_threads=1, form=FORM_FP64):
        lib = load_library()
        x = np.ascontiguousarray(x)
        if x.dtype not in (np.float32, np.float64):
            x = x.astype(np.float64)
        i = np.ascontiguousarray(i, dtype=np.int32)
        p = np.ascontiguousarray(p, dtype=np.int64)
        h = ctypes.c_void_p()
        vt = VALUE_F64 if x.dtype == np.float64 else VALUE_F32
        _check(lib.irlba_gb300_matrix_create_sparse(nrow, ncol, _vptr(x), vt, _vptr(i), _vptr(p),
                                                    int(bool(column_major)), form, ctypes.byref(h)))
        super().__init__(h.value, nrow, ncol, form)
        self.num_threads = num_threads

    def layout(self):
        lib = load_library()
        nnz = ctypes.c_int64()
        vb, im, ia, pm, pa = (ctypes.c_int32() for _ in range(5))
        _check(lib.irlba_gb300_matrix_layout(self._h, ctypes.byref(nnz), ctypes.byref(vb), ctypes.byref(im),
                                             ctypes.byref(ia), ctypes.byref(pm), ctypes.byref(pa)))
        return {"nnz": nnz.value, "value_bytes": vb.value, "index_bytes_mul": im.value,
                "index_bytes_adj": ia.value, "panels_mul": pm.value, "panels_adj": pa.value}


def compressed_arrays(matrix):
    """(values, indices, pointers, column_major) of a scipy.sparse matrix in the
    C ABI's layout: CSC stays column-major and CSR row-major (any other sparse
    format is read as CSR); duplicate entries are summed and indices sorted
    within each row or column, as Eigen's compressed storage has them."""
    import scipy.sparse as sp
    if not sp.issparse(matrix):
        raise TypeError("not a scipy.sparse matrix")
    column_major = matrix.format == "csc"
    m = matrix.tocsc() if column_major else matrix.tocsr()
    m = m.copy()
    m.sum_duplicates()
    m.sort_indices()
    values = np.ascontiguousarray(m.data)
    if values.dtype not in (np.float32, np.float64):
        values = values.astype(np.float64)
    return (values, np.ascontiguousarray(m.indices, dtype=np.int32), np.ascontiguousarray(m.indptr, dtype=np.int64),
            column_major)


class SimpleMatrix(Matrix):
    """irlba::SimpleMatrix over a dense matrix or a sparse one
    (Matrix/simple.hpp:124-178 wraps either Eigen type); scipy.sparse input is
    stored in the same device layout as ParallelSparseMatrix."""

    def __init__(self, dense, form=FORM_FP64):
        lib = load_library()
        if _is_scipy_sparse(dense):
            x, i, p, column_major = compressed_arrays(dense)
            nrow, ncol = dense.shape
            h = ctypes.c_void_p()
            vt = VALUE_F64 if x.dtype == np.float64 else VALUE_F32
            _check(lib.irlba_gb300_matrix_create_sparse(nrow, ncol, _vptr(x), vt, _vptr(i), _vptr(p),
                                                        int(column_major), form, ctypes.byref(h)))
            super().__init__(h.value, nrow, ncol, form)
            return
        a = np.asarray(dense)
        if a.dtype not in (np.float32, np.float64):
            a = a.astype(np.float64)
        if a.flags.f_contiguous:
            row_major, buf, ld = 0, a, a.shape[0]
        else:
            a = np.ascontiguousarray(a)
            row_major, buf, ld = 1, a, a.shape[1]
        h = ctypes.c_void_p()
        vt = VALUE_F64 if buf.dtype == np.float64 else VALUE_F32
        _check(lib.irlba_gb300_matrix_create_dense(a.shape[0], a.shape[1], _vptr(buf), vt, max(ld, 1), row_major,
                                                   form, ctypes.byref(h)))
        super().__init__(h.value, a.shape[0], a.shape[1], form)


# irlba_gb300_host_product / irlba_gb300_device_product (include/irlba_gb300.h).
HOST_PRODUCT = ctypes.CFUNCTYPE(ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_double),
                                ctypes.POINTER(ctypes.c_double))
DEVICE_PRODUCT = ctypes.CFUNCTYPE(ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p)


class OperatorMatrix(Matrix):
    """A user-defined irlba::Matrix (Matrix/interface.hpp:141-223) whose products
    are Python callables on FP64 numpy vectors: multiply(x) returns A @ x (x of
    length ncol) and adjoint_multiply(y) returns A.T @ y. The IRLBA loop stays on
    the device; each product copies its vectors to the host and back (correct,
    not fast). Centring and scaling decorators may wrap it; pca() may not."""

    def __init__(self, nrow, ncol, multiply, adjoint_multiply, form=FORM_FP64):
        lib = load_library()

        def product(_user, adjoint, x, y):
            try:
                n_in, n_out = (nrow, ncol) if adjoint else (ncol, nrow)
                xa = np.ctypeslib.as_array(x, shape=(n_in,)).copy()
                res = np.asarray((adjoint_multiply if adjoint else multiply)(xa), dtype=np.float64)
                if res.shape != (n_out,):
                    raise ValueError("product returned shape %s, expected (%d,)" % (res.shape, n_out))
                np.ctypeslib.as_array(y, shape=(n_out,))[:] = res
                return 0
            except BaseException as exc:  # reported through the engine's status
                _callback_state.error = exc
                return 1

        cb = HOST_PRODUCT(product)
        h = ctypes.c_void_p()
        _check(lib.irlba_gb300_matrix_create_host_operator(nrow, ncol, ctypes.cast(cb, ctypes.c_void_p), None, form,
                                                           ctypes.byref(h)))
        super().__init__(h.value, nrow, ncol, form, keep=[cb])


class DeviceOperatorMatrix(Matrix):
    """A user-defined irlba::Matrix whose products run on the device, e.g. a
    residual matrix that is never stored. `product(adjoint, x_ptr, y_ptr,
    stream)` enqueues y = A x (adjoint False; x of length ncol) or y = A.T x on
    the cudaStream_t `stream` (an int) and returns; x and y are device
    addresses of float64 vectors (FORM_FP64) or float32 vectors
    (FORM_FP32_FP64STEPS). `product` may instead be the address of a C function
    with the irlba_gb300_device_product signature, with `user` its first
    argument."""

    def __init__(self, nrow, ncol, product, form=FORM_FP64, user=None):
        lib = load_library()
        keep = []
        if callable(product):
            def tramp(_user, adjoint, x, y, stream):
                try:
                    product(bool(adjoint), x or 0, y or 0, stream or 0)
                    return 0
                except BaseException as exc:  # reported through the engine's status
                    _callback_state.error = exc
                    return 1
            cb = DEVICE_PRODUCT(tramp)
            keep.append(cb)
            fptr = ctypes.cast(cb, ctypes.c_void_p)
        else:
            fptr = ctypes.c_void_p(int(product))
        h = ctypes.c_void_p()
        _check(lib.irlba_gb300_matrix_create_device_operator(nrow, ncol, fptr, ctypes.c_void_p(user or 0), form,
                                                             ctypes.byref(h)))
        super().__init__(h.value, nrow, ncol, form, keep=keep)


class CenteredMatrix(Matrix):
    """irlba::CenteredMatrix(matrix, center) (Matrix/centered.hpp:152)."""

    def __init__(self, matrix, center):
        c = np.ascontiguousarray(center, dtype=np.float64)
        if c.shape != (matrix.cols(),):
            raise ValueError("center must have length cols()")
        h = ctypes.c_void_p()
        _check(load_library().irlba_gb300_matrix_center(matrix.handle, _dptr(c), ctypes.byref(h)))
        super().__init__(h.value, matrix.rows(), matrix.cols(), matrix.form, keep=[matrix])


class ScaledMatrix(Matrix):
    """irlba::ScaledMatrix(matrix, scale, column, divide) (Matrix/scaled.hpp:420)."""

    def __init__(self, matrix, scale, column, divide):
        s = np.ascontiguousarray(scale, dtype=np.float64)
        want = matrix.cols() if column else matrix.rows()
        if s.shape != (want,):
            raise ValueError("scale has the wrong length")
        h = ctypes.c_void_p()
        _check(load_library().irlba_gb300_matrix_scale(matrix.handle, _dptr(s), int(bool(column)),
                                                       int(bool(divide)), ctypes.byref(h)))
        super().__init__(h.value, matrix.rows(), matrix.cols(), matrix.form, keep=[matrix])


def compute(matrix, number, options=None):
    """irlba::compute(matrix, number, options) (compute.hpp:403-410)."""
    options = options or Options()
    keep = []
    o = options._to_c(keep)
    m, n = matrix.rows(), matrix.cols()
    cap = max(min(number, min(m, n)), 0)
    U = np.empty((cap, m))  # column-major m x cap, as the C ABI writes it
    V = np.empty((cap, n))
    D = np.zeros(max(cap, 1))
    num = ctypes.c_int64()
    conv = ctypes.c_int32()
    iters = ctypes.c_int32()
    st = Stats()
    _check(load_library().irlba_gb300_compute(matrix.handle, number, ctypes.byref(o), _dptr(U), _dptr(V), _dptr(D),
                                              ctypes.byref(num), ctypes.byref(conv), ctypes.byref(iters),
                                              ctypes.byref(st)))
    r = num.value
    return Results(U=U[:r].T, V=V[:r].T, D=D[:r].copy(), iterations=iters.value,
                   converged=bool(conv.value), stats=_stats_dict(st))


def compute_simple(matrix, number, options=None, form=FORM_FP64):
    """irlba::compute_simple(matrix, number, options) (compute.hpp:426-433)."""
    return compute(SimpleMatrix(matrix, form=form), number, options)


def pca(matrix, center, scale, number, options=None):
    """irlba::pca(matrix, center, scale, number, options) (pca.hpp:197-204).

    `matrix` is an undecorated ParallelSparseMatrix or SimpleMatrix (rows are
    observations, columns are features), or a numpy array or scipy.sparse
    matrix (wrapped in a SimpleMatrix)."""
    if isinstance(matrix, np.ndarray) or _is_scipy_sparse(matrix):
        matrix = SimpleMatrix(matrix)
    options = options or Options()
    keep = []
    o = options._to_c(keep)
    m, n = matrix.rows(), matrix.cols()
    cap = max(min(number, min(m, n)), 0)
    S = np.empty((cap, m))  # column-major m x cap, as the C ABI writes it
    R = np.empty((cap, n))
    var = np.zeros(max(cap, 1))
    c_out = np.zeros(max(n, 1))
    s_out = np.zeros(max(n, 1))
    num = ctypes.c_int64()
    conv = ctypes.c_int32()
    iters = ctypes.c_int32()
    st = Stats()
    _check(load_library().irlba_gb300_pca(matrix.handle, int(bool(center)), int(bool(scale)), number,
                                          ctypes.byref(o), _dptr(S), _dptr(R), _dptr(var), ctypes.byref(num),
                                          ctypes.byref(conv), ctypes.byref(iters), _dptr(c_out), _dptr(s_out),
                                          ctypes.byref(st)))
    r = num.value
    return PcaResults(scores=S[:r].T, rotation=R[:r].T, variances=var[:r].copy(),
                      iterations=iters.value, converged=bool(conv.value),
                      center=c_out[:n].copy() if center else None, scale=s_out[:n].copy() if scale else None,
                      stats=_stats_dict(st))


def update_k_device(quads):
    """The device restart step's update_k (compute.hpp:78-111) for an (n, 4)
    array of (k, requested, n_converged, work); returns the n next k values."""
    q = np.ascontiguousarray(np.asarray(quads, dtype=np.int32).reshape(-1, 4))
    out = np.zeros(q.shape[0], dtype=np.int32)
    _check(load_library().irlba_gb300_update_k_device(ctypes.c_void_p(q.ctypes.data), q.shape[0],
                                                      ctypes.c_void_p(out.ctypes.data)))
    return out


def device_count():
    return load_library().irlba_gb300_device_count()


def set_device_ingest(on):
    """Build sparse matrices' device layout on the GPU (default) or on the host."""
    load_library().irlba_gb300_set_device_ingest(int(bool(on)))


def set_spmv_shape(shape):
    """Launch shape of the sparse products of FP32-form matrices created
    afterwards: 0 = 256-thread CTAs, 1 = 256 threads six per SM, 2 (default) =
    512 threads three per SM."""
    load_library().irlba_gb300_set_spmv_shape(int(shape))


def set_rotation_engine(engine):
    """Engine of the restart rotations (w, k <= 64) of later compute calls:
    1 = tensor cores (default), 0 = CUDA cores."""
    load_library().irlba_gb300_set_rotation_engine(int(engine))


def set_value_coding(on):
    """Dictionary coding of FP32-form sparse matrices created afterwards: at
    most 2,048 distinct values are kept as 16-bit codes into a table of the
    exact values for the products (off by default; results unchanged)."""
    load_library().irlba_gb300_set_value_coding(int(bool(on)))


def set_staging(min_bytes=16 << 20, slice_bytes=8 << 20):
    """Copies of pageable host memory of at least `min_bytes` (< 0: never) go
    through pinned staging buffers of `slice_bytes`, filled by host threads."""
    load_library().irlba_gb300_set_staging(int(min_bytes), int(slice_bytes))


def set_profiling(on):
    load_library().irlba_gb300_set_profiling(int(bool(on)))


def last_profile():
    ms = (ctypes.c_double * 6)()
    launches = (ctypes.c_int64 * 6)()
    load_library().irlba_gb300_last_profile(ms, launches)
    names = ["spmv_mul", "spmv_adj", "cgs", "restart", "rotate", "other"]
    return {n: {"ms": ms[i], "launches": launches[i]} for i, n in enumerate(names)}


def launch_count():
    return load_library().irlba_gb300_launch_count()


def transfer_bytes():
    """(host-to-device, device-to-host) bytes copied by the library so far."""
    h, d = ctypes.c_int64(), ctypes.c_int64()
    load_library().irlba_gb300_transfer_bytes(ctypes.byref(h), ctypes.byref(d))
    return h.value, d.value


class Batch:
    """Batched form (no counterpart in the reference): many sparse matrices on
    the device, each solved as irlba::pca(matrix_j, center, scale, number,
    options) would solve it, in one persistent launch replayed from a captured
    CUDA graph. `matrices` is a list of (nrow, ncol, x, i, p) compressed
    matrices sharing `column_major` (the ParallelSparseMatrix arguments)."""

    def __init__(self, matrices, column_major):
        lib = load_library()
        self.count = len(matrices)
        f64 = any(np.asarray(mx[2]).dtype == np.float64 for mx in matrices)
        dt = np.float64 if f64 else np.float32
        self._keep = []
        nrow = np.array([int(mx[0]) for mx in matrices], dtype=np.int64)
        ncol = np.array([int(mx[1]) for mx in matrices], dtype=np.int64)
        vals = (ctypes.c_void_p * max(self.count, 1))()
        idxs = (ctypes.c_void_p * max(self.count, 1))()
        ptrs = (ctypes.c_void_p * max(self.count, 1))()
        for j, (_, _, x, i, pp) in enumerate(matrices):
            x = np.ascontiguousarray(x, dtype=dt)
            i = np.ascontiguousarray(i, dtype=np.int32)
            pp = np.ascontiguousarray(pp, dtype=np.int64)
            self._keep += [x, i, pp]
            vals[j], idxs[j], ptrs[j] = x.ctypes.data, i.ctypes.data, pp.ctypes.data
        self.nrow, self.ncol = nrow, ncol
        h = ctypes.c_void_p()
        _check(lib.irlba_gb300_batch_create(self.count, _vptr(nrow), _vptr(ncol), vals,
                                            VALUE_F64 if f64 else VALUE_F32, idxs, ptrs,
                                            int(bool(column_major)), ctypes.byref(h)))
        self._keep = []  # the library holds its own copies
        self._h = h
        self._number = 0
        self._center = self._scale = False

    def close(self):
        if self._h and self._h.value:
            load_library().irlba_gb300_batch_destroy(self._h)
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def groups(self):
        gm = np.zeros(max(self.count, 1), dtype=np.int32)
        ga = np.zeros(max(self.count, 1), dtype=np.int32)
        _check(load_library().irlba_gb300_batch_groups(self._h, _vptr(gm), _vptr(ga)))
        return gm[:self.count], ga[:self.count]

    def set_groups(self, group_mul=None, group_adj=None):
        gm = None if group_mul is None else np.ascontiguousarray(group_mul, dtype=np.int32)
        ga = None if group_adj is None else np.ascontiguousarray(group_adj, dtype=np.int32)
        _check(load_library().irlba_gb300_batch_set_groups(self._h, None if gm is None else _vptr(gm),
                                                           None if ga is None else _vptr(ga)))

    def set_team(self, team, joint=-1):
        """CTAs per team (1, 2, 4; 0 = automatic) and how many of the largest
        matrices a team solves together (-1 = automatic)."""
        _check(load_library().irlba_gb300_batch_set_team(self._h, int(team), int(joint)))

    def tune(self, repeats=3, stream=None):
        _check(load_library().irlba_gb300_batch_tune(self._h, repeats, stream))

    def pca(self, center, scale, number, options=None, stream=None):
        """Solve every matrix; returns the call's statistics (a dict)."""
        options = options or Options()
        keep = []
        o = options._to_c(keep)
        st = BatchStats()
        _check(load_library().irlba_gb300_batch_pca(self._h, int(bool(center)), int(bool(scale)), number,
                                                    ctypes.byref(o), ctypes.byref(st), stream))
        self._number, self._center, self._scale = number, bool(center), bool(scale)
        return {f: getattr(st, f) for f, _ in BatchStats._fields_ if f != "reserved0"}

    def result(self, j):
        """PcaResults of matrix j from the last pca() call (info in .stats)."""
        if not 0 <= j < self.count:
            # The library reports the error (index or missing results).
            _check(load_library().irlba_gb300_batch_result(self._h, j, None, None, None, None, None, None))
        m, n = int(self.nrow[j]), int(self.ncol[j])
        r = max(min(self._number, min(m, n)), 0)
        S = np.empty((max(self._number, 1), m))
        R = np.empty((max(self._number, 1), n))
        var = np.zeros(max(self._number, 1))
        c_out = np.zeros(max(n, 1))
        s_out = np.zeros(max(n, 1))
        inf = BatchInfo()
        _check(load_library().irlba_gb300_batch_result(self._h, j, _dptr(S), _dptr(R), _dptr(var), _dptr(c_out),
                                                       _dptr(s_out), ctypes.byref(inf)))
        info = {f: getattr(inf, f) for f, _ in BatchInfo._fields_}
        return PcaResults(scores=S[:r].T, rotation=R[:r].T, variances=var[:r].copy(),
                          iterations=inf.iterations, converged=bool(inf.converged),
                          center=c_out[:n].copy() if self._center else None,
                          scale=s_out[:n].copy() if self._scale else None, stats=info)
