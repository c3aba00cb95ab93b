"""Dictionary-coded values of FP32-form sparse matrices, through the C ABI.

A matrix with at most 2,048 distinct FP32 values keeps each value as a 16-bit
code into a table of the exact values for the products; the products must be
those of the stored values (checked against an FP64 product of the FP32 values
at the FP32 form's 1e-5 and against the same matrix without coding at 1e-6,
the two differing only in the FP32 summation order), and a PCA on the coded
matrix must give the uncoded one's results. Matrices with more distinct values
keep the plain layout. Coding is off by default and switched on per matrix here."""
import numpy as np
import pytest

from conftest import principal_sines

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def _matrix(engine, nr, nc, values, seed, coded, column_major=True, density=0.1):
    """A compressed sparse matrix whose entries are drawn from `values`."""
    rng = np.random.default_rng(seed)
    mask = rng.random((nr, nc)) < density
    dense = np.where(mask, rng.choice(values, size=(nr, nc)), 0.0).astype(np.float32)
    if column_major:
        ptr = np.concatenate([[0], np.cumsum(mask.sum(axis=0))]).astype(np.int64)
        idx = np.concatenate([np.nonzero(mask[:, c])[0] for c in range(nc)]).astype(np.int32)
        val = np.concatenate([dense[mask[:, c], c] for c in range(nc)]).astype(np.float32)
    else:
        ptr = np.concatenate([[0], np.cumsum(mask.sum(axis=1))]).astype(np.int64)
        idx = np.concatenate([np.nonzero(mask[r])[0] for r in range(nr)]).astype(np.int32)
        val = np.concatenate([dense[r, mask[r]] for r in range(nr)]).astype(np.float32)
    engine.set_value_coding(coded)
    try:
        m = engine.ParallelSparseMatrix(nr, nc, val, idx, ptr, column_major, form=engine.FORM_FP32_FP64STEPS)
    finally:
        engine.set_value_coding(False)
    return m, dense.astype(np.float64), (val, idx, ptr)


@pytest.mark.parametrize("ndistinct,expect_coded", [(1, True), (300, True), (2048, True), (2049, False)])
@pytest.mark.parametrize("column_major", [True, False])
def test_coded_products(engine, ndistinct, expect_coded, column_major):
    rng = np.random.default_rng(ndistinct)
    values = np.unique(np.log1p(rng.permutation(np.arange(1, 100000))[:ndistinct]).astype(np.float32))
    assert len(values) == ndistinct
    nr, nc = 3000, 40000   # the adjoint gathers over three panels of x
    m, dense, _ = _matrix(engine, nr, nc, values, seed=ndistinct + column_major, coded=True,
                          column_major=column_major, density=0.02)
    assert (m.layout()["value_bytes"] == 2) == expect_coded
    plain, _, _ = _matrix(engine, nr, nc, values, seed=ndistinct + column_major, coded=False,
                          column_major=column_major, density=0.02)
    assert plain.layout()["value_bytes"] == 4
    v = rng.standard_normal(nc)
    w = rng.standard_normal(nr)
    for mat in (m, plain):
        assert _rel(mat.multiply(v), dense @ v) < 1e-5
        assert _rel(mat.adjoint_multiply(w), dense.T @ w) < 1e-5
    assert _rel(m.multiply(v), plain.multiply(v)) < 1e-6
    assert _rel(m.adjoint_multiply(w), plain.adjoint_multiply(w)) < 1e-6


def test_coded_signed_zero_and_negative_values(engine):
    # -0.0 and 0.0 are distinct bit patterns (both stored entries), negative
    # values and values of very different magnitude share one dictionary.
    values = np.array([-0.0, 0.0, -3.5, 1e-30, 7.25e20, 2.0, -1e-3], dtype=np.float32)
    m, dense, _ = _matrix(engine, 800, 5000, values, seed=5, coded=True)
    assert m.layout()["value_bytes"] == 2
    v = np.random.default_rng(6).standard_normal(5000)
    w = np.random.default_rng(7).standard_normal(800)
    got, ref = m.multiply(v), dense @ v
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(dense) @ np.abs(v), 1e-300)) < 1e-5
    got, ref = m.adjoint_multiply(w), dense.T @ w
    assert np.max(np.abs(got - ref) / np.maximum(np.abs(dense).T @ np.abs(w), 1e-300)) < 1e-5


def test_coded_pca_matches_plain(engine):
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_pca_input(500, 30000, 0.1, seed=11, dtype=np.float32, cell_major=False)
    init = datagen.start_vector(inp.ncol)
    res = []
    for coded in (True, False):
        engine.set_value_coding(coded)
        try:
            mat = engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major,
                                              form=engine.FORM_FP32_FP64STEPS)
        finally:
            engine.set_value_coding(False)
        assert mat.layout()["value_bytes"] == (2 if coded else 4)
        res.append(engine.pca(mat, True, True, 10, engine.Options(initial=init)))
    a, b = res
    np.testing.assert_allclose(a.variances, b.variances, rtol=1e-6)
    assert principal_sines(a.rotation, b.rotation).max() < 1e-4
