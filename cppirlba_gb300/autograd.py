"""Differentiation form: the truncated SVD and pca()'s sparse SVD as torch
autograd operations, backed by libtorch C++ torch::autograd::Function classes
(csrc/torch_ops.cpp) over the engine's C ABI.

truncated_svd(A, k)  -> (U, S, V) of a dense CUDA matrix (FP32 uses the
    FP32+FP64-steps form, FP64 the plain form); backward: the truncated-SVD
    adjoint (F-matrix terms, plus the orthogonal-complement terms solved by
    shifted conjugate gradients to relative residual cg_tol: by default 1e-8
    for FP32 input and 1e-12 for FP64; cg_tol < 0 for the rank-k projection
    terms).
sparse_pca_svd(values, pointers, indices, nrow, ncol, column_major, center,
    scale, k) -> (U, S, V, center, scale) of pca()'s centred/scaled operator of
    a compressed sparse matrix; backward: the gradient on the stored values
    (SDDMM), through the centring and scaling and, with statistics=True, the
    column statistics' own dependence on the values.
pca scores and variances follow from (U, S) as in pca.hpp:130-136:
scores = U * S, variances = S**2 / (nrow - 1).
"""
import importlib.util
import os

import torch

from . import load_library

_ext = None


def load_extension():
    """Import the libtorch extension (building it first if it is absent)."""
    global _ext
    if _ext is None:
        load_library()
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "_irlba_torch.so")
        if not os.path.exists(path):
            from . import build as _build
            _build.build(torch_ext=True)
        spec = importlib.util.spec_from_file_location("_irlba_torch", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        _ext = mod
    return _ext


def _cg_tol(cg_tol, dtype):
    # The complement solves need no more accuracy than the forward carries.
    if cg_tol is not None:
        return float(cg_tol)
    return 1e-8 if dtype == torch.float32 else 1e-12


def truncated_svd(A, k, tol=1e-10, seed=5489, cg_tol=None, cg_max_iter=5000):
    return load_extension().truncated_svd(A, int(k), float(tol), int(seed), _cg_tol(cg_tol, A.dtype),
                                          int(cg_max_iter))


def sparse_pca_svd(values, pointers, indices, nrow, ncol, column_major, center, scale, k, tol=1e-10, seed=5489,
                   cg_tol=None, cg_max_iter=5000, statistics=True):
    pointers = torch.as_tensor(pointers, dtype=torch.int64).contiguous().cpu()
    indices = torch.as_tensor(indices, dtype=torch.int32).contiguous().cpu()
    return load_extension().sparse_pca_svd(values, pointers, indices, int(nrow), int(ncol), bool(column_major),
                                           bool(center), bool(scale), int(k), float(tol), int(seed),
                                           _cg_tol(cg_tol, values.dtype), int(cg_max_iter), bool(statistics))
