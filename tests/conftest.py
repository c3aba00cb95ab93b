import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine through the C ABI")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def engine():
    import cppirlba_gb300 as eng
    eng.load_library()
    if eng.device_count() < 1:
        pytest.fail("GPU test collected but no CUDA device is visible")
    return eng


def normal_matrix(nr, nc, seed=42):
    return np.random.default_rng(seed).standard_normal((nr, nc))


def simulate_compressed_sparse(nr, nc, density=0.2, seed=None):
    """Compressed-sparse-column test matrix in the spirit of the reference's
    tests/src/sparse.h:18-44 (density 0.2, N(0, 1) values, seed nr*nc)."""
    rng = np.random.default_rng(nr * nc if seed is None else seed)
    mask = rng.random((nr, nc)) < density
    vals = rng.standard_normal((nr, nc))
    ptr = [0]
    idx, val = [], []
    for c in range(nc):
        rows = np.nonzero(mask[:, c])[0]
        idx.extend(rows.tolist())
        val.extend(vals[rows, c].tolist())
        ptr.append(len(idx))
    dense = np.where(mask, vals, 0.0)
    return dense, np.array(val, dtype=np.float64), np.array(idx, dtype=np.int32), np.array(ptr, dtype=np.int64)


def to_csr(dense):
    ptr = [0]
    idx, val = [], []
    for r in range(dense.shape[0]):
        cols = np.nonzero(dense[r])[0]
        idx.extend(cols.tolist())
        val.extend(dense[r, cols].tolist())
        ptr.append(len(idx))
    return np.array(val, dtype=np.float64), np.array(idx, dtype=np.int32), np.array(ptr, dtype=np.int64)


def same_same(a, b, tol):
    """compare.h:7-9 of the reference's tests."""
    return abs(a - b) <= (abs(a) + abs(b)) * tol


def principal_sines(A, B):
    """Sines of the principal angles between the column spans of A and B."""
    qa, _ = np.linalg.qr(A)
    qb, _ = np.linalg.qr(B)
    resid = qa - qb @ (qb.T @ qa)
    return np.linalg.svd(resid, compute_uv=False)


def column_sines(A, B):
    """Per-column sine of the angle between A[:, j] and B[:, j] (sign-agnostic)."""
    out = []
    for j in range(A.shape[1]):
        a = A[:, j] / np.linalg.norm(A[:, j])
        b = B[:, j] / np.linalg.norm(B[:, j])
        out.append(float(np.linalg.norm(a - (a @ b) * b)))
    return np.array(out)
