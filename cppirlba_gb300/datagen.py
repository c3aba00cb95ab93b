"""Seeded synthetic inputs standing in for the single-cell count matrices that
CppIrlba's sparse PCA path serves (no public dataset is used by the reference).

Sparse matrices come from the multithreaded C++ generator in csrc/datagen.cpp
(value model: Bernoulli(density) presence, per-gene mean LogNormal(mu, sigma),
negative-binomial counts with dispersion phi conditioned on >= 1, value =
log1p(count)). Dense planted-spectrum matrices use numpy's PCG64 generator.

Workloads (rows of every PCA input are observations = cells):
  dense_planted   1000 x 200 FP64, singular values 100, 90, ..., 10 on orthonormal
                  factors from the QR of seeded Gaussian matrices, plus iid N(0, 1).
  scrna_csc_20k   20,000 genes x 50,000 cells, density 0.05, FP64 values; stored
                  CSC genes x cells = CSR cells x genes (pca input, column_major=0).
  scrna_csr_2k    2,000 genes x 1.3M cells, density 0.10, FP32 values; stored CSR
                  genes x cells = CSC cells x genes (pca input, column_major=1).
  batched         256 matrices of 2,000 genes x n_j cells, n_j = clamp(round(
                  LogNormal(log 5000, 1.0)), 200, 50000), density 0.08, FP32.
  adjoint_dense   4096 x 1024 FP32, sigma_i = 50 / i on orthonormal factors plus
                  N(0, 0.01^2) noise (0.01 read as the standard deviation).
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libirlba_gb300_datagen.so")
_lib = None

# Value model constants of the single-cell generator.
GENE_MEAN_MU = -1.0
GENE_MEAN_SIGMA = 1.5
DISPERSION = 0.5


def _declare(lib):
    """Declares the generator's C entry points on a loaded library."""
    i64, dbl, u64, P = ctypes.c_int64, ctypes.c_double, ctypes.c_uint64, ctypes.c_void_p
    lib.irlba_gb300_datagen_counts.restype = i64
    lib.irlba_gb300_datagen_counts.argtypes = [i64, i64, dbl, u64, ctypes.c_int, P]
    lib.irlba_gb300_datagen_fill.restype = None
    lib.irlba_gb300_datagen_fill.argtypes = [i64, i64, dbl, dbl, dbl, dbl, u64, ctypes.c_int, P, P, P, ctypes.c_int]
    lib.irlba_gb300_datagen_gene_means.restype = None
    lib.irlba_gb300_datagen_gene_means.argtypes = [i64, dbl, dbl, u64, P]
    lib.irlba_gb300_transpose_compressed.restype = None
    lib.irlba_gb300_transpose_compressed.argtypes = [i64, i64, P, P, P, ctypes.c_int, P, P, P]
    return lib


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        from . import build as _build
        _build.build()
    _lib = _declare(ctypes.CDLL(_LIB_PATH))
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def scrna_gene_major(genes, cells, density, seed, dtype=np.float32, threads=None, lib=None):
    """Gene-major compressed matrix (genes x cells): (ptr int64, idx int32 cell, values).
    lib: another loaded library that exports the same generator (default: this
    package's generator library)."""
    lib = _declare(lib) if lib is not None else _load()
    threads = threads or os.cpu_count() or 1
    ptr = np.zeros(genes + 1, dtype=np.int64)
    nnz = lib.irlba_gb300_datagen_counts(genes, cells, density, seed, threads, _p(ptr))
    idx = np.empty(nnz, dtype=np.int32)
    val = np.empty(nnz, dtype=dtype)
    lib.irlba_gb300_datagen_fill(genes, cells, density, GENE_MEAN_MU, GENE_MEAN_SIGMA, DISPERSION, seed, threads,
                                 _p(ptr), _p(idx), _p(val), val.itemsize)
    return ptr, idx, val


def transpose_compressed(primary, secondary, ptr, idx, val, lib=None):
    """(secondary x primary) compressed transpose, indices sorted."""
    lib = _declare(lib) if lib is not None else _load()
    tptr = np.zeros(secondary + 1, dtype=np.int64)
    tidx = np.empty(idx.shape[0], dtype=np.int32)
    tval = np.empty(val.shape[0], dtype=val.dtype)
    lib.irlba_gb300_transpose_compressed(primary, secondary, _p(ptr), _p(idx), _p(val), val.itemsize, _p(tptr),
                                         _p(tidx), _p(tval))
    return tptr, tidx, tval


class SparseInput:
    """A PCA input: nrow observations x ncol features, compressed in `column_major`
    order (ptr over the primary dimension)."""

    def __init__(self, nrow, ncol, ptr, idx, val, column_major):
        self.nrow, self.ncol = nrow, ncol
        self.ptr, self.idx, self.val = ptr, idx, val
        self.column_major = column_major

    @property
    def nnz(self):
        return int(self.ptr[-1])

    def to_dense(self):
        out = np.zeros((self.nrow, self.ncol))
        prim = self.ncol if self.column_major else self.nrow
        for p in range(prim):
            s, e = self.ptr[p], self.ptr[p + 1]
            if self.column_major:
                out[self.idx[s:e], p] = self.val[s:e]
            else:
                out[p, self.idx[s:e]] = self.val[s:e]
        return out


def scrna_pca_input(genes, cells, density, seed, dtype, cell_major, lib=None):
    """Cells x genes PCA input. cell_major=True gives CSR cells x genes (the
    genes x cells CSC layout); False gives CSC cells x genes (genes x cells CSR)."""
    ptr, idx, val = scrna_gene_major(genes, cells, density, seed, dtype=dtype, lib=lib)
    if cell_major:
        tptr, tidx, tval = transpose_compressed(genes, cells, ptr, idx, val, lib=lib)
        return SparseInput(cells, genes, tptr, tidx, tval, column_major=False)
    return SparseInput(cells, genes, ptr, idx, val, column_major=True)


def scrna_csc_20k(seed=2, genes=20000, cells=50000, density=0.05):
    return scrna_pca_input(genes, cells, density, seed, np.float64, cell_major=True)


def scrna_csr_2k(seed=3, genes=2000, cells=1300000, density=0.10, dtype=np.float32):
    return scrna_pca_input(genes, cells, density, seed, dtype, cell_major=False)


def dense_planted(nr=1000, nc=200, rank=10, seed=1):
    rng = np.random.default_rng(seed)
    U0, _ = np.linalg.qr(rng.standard_normal((nr, rank)))
    V0, _ = np.linalg.qr(rng.standard_normal((nc, rank)))
    sv = np.arange(rank, 0, -1, dtype=np.float64) * 10.0
    return (U0 * sv) @ V0.T + rng.standard_normal((nr, nc))


def batched_sizes(count=256, seed=4, lo=200, hi=50000, median=5000.0, sigma=1.0):
    rng = np.random.default_rng(seed)
    n = np.round(np.exp(np.log(median) + sigma * rng.standard_normal(count)))
    return np.clip(n, lo, hi).astype(np.int64)


def scrna_batch(sizes, genes=2000, density=0.08, seed=4, dtype=np.float32, cell_major=False):
    """One cells x genes PCA input per entry of `sizes` (cells), same value model
    as scrna_pca_input; matrix j uses seed + 1000 + j."""
    return [scrna_pca_input(genes, int(c), density, seed + 1000 + j, dtype, cell_major)
            for j, c in enumerate(sizes)]


def adjoint_dense(nr=4096, nc=1024, seed=5, noise_sd=0.01, dtype=np.float32):
    """Planted spectrum sigma_i = 50 / i plus iid N(0, noise_sd^2) noise."""
    rng = np.random.default_rng(seed)
    k = min(nr, nc)
    U0, _ = np.linalg.qr(rng.standard_normal((nr, k)))
    V0, _ = np.linalg.qr(rng.standard_normal((nc, k)))
    sv = 50.0 / np.arange(1, k + 1)
    return ((U0 * sv) @ V0.T + noise_sd * rng.standard_normal((nr, nc))).astype(dtype)


def start_vector(n, seed=12345):
    """Seeded start vector shared by the GPU runs and the oracle (Options.initial)."""
    return np.random.default_rng(seed).standard_normal(n)
