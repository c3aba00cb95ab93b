"""Device-side ingestion builds the same gather plans as the host builder:
layouts, products and whole solves agree bit for bit, for both storage
orders, both precision forms, single- and multi-panel layouts and the
unstaged (very sparse) layout; unsorted rows fall back to the host builder."""
import numpy as np
import pytest

from conftest import simulate_compressed_sparse, to_csr

pytestmark = pytest.mark.gpu


def _both(engine, build):
    engine.set_device_ingest(True)
    try:
        dev = build()
        engine.set_device_ingest(False)
        host = build()
    finally:
        engine.set_device_ingest(True)
    return dev, host


def _same_products(engine, a, b, nr, nc, seed=1):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(nc)
    y = rng.standard_normal(nr)
    np.testing.assert_array_equal(a.multiply(x), b.multiply(x))
    np.testing.assert_array_equal(a.adjoint_multiply(y), b.adjoint_multiply(y))


@pytest.mark.parametrize("form", ["fp64", "fp32"])
@pytest.mark.parametrize("column_major", [True, False])
@pytest.mark.parametrize("nr,nc,density", [(300, 120, 0.2), (40000, 90, 0.05), (70, 36000, 0.08),
                                           (120000, 40, 0.0004)])
def test_device_and_host_plans_agree(engine, form, column_major, nr, nc, density):
    f = engine.FORM_FP64 if form == "fp64" else engine.FORM_FP32_FP64STEPS
    dense, x, i, p = simulate_compressed_sparse(nr, nc, density=density, seed=nr + nc)
    if not column_major:
        x, i, p = to_csr(dense)

    def build():
        return engine.ParallelSparseMatrix(nr, nc, x, i, p, column_major, form=f)

    dev, host = _both(engine, build)
    assert dev.layout() == host.layout()
    _same_products(engine, dev, host, nr, nc)
    if min(nr, nc) > 12:
        a = engine.compute(dev, 4, engine.Options(seed=3))
        b = engine.compute(host, 4, engine.Options(seed=3))
        np.testing.assert_array_equal(a.D, b.D)
        np.testing.assert_array_equal(a.U, b.U)
        np.testing.assert_array_equal(a.V, b.V)


def test_scrna_pca_device_ingest_matches_host(engine):
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_pca_input(500, 30000, 0.1, seed=29, dtype=np.float32, cell_major=False)

    def build():
        return engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major,
                                           form=engine.FORM_FP32_FP64STEPS)

    dev, host = _both(engine, build)
    a = engine.pca(dev, True, True, 8, engine.Options(seed=11))
    b = engine.pca(host, True, True, 8, engine.Options(seed=11))
    np.testing.assert_array_equal(a.variances, b.variances)
    np.testing.assert_array_equal(a.rotation, b.rotation)
    np.testing.assert_array_equal(a.center, b.center)
    np.testing.assert_array_equal(a.scale, b.scale)


def test_unsorted_rows_and_index_errors(engine):
    dense, x, i, p = simulate_compressed_sparse(200, 60, seed=5)
    # Reverse the order inside every column: valid input, unsorted rows.
    xs, is_ = x.copy(), i.copy()
    for c in range(60):
        b, e = p[c], p[c + 1]
        xs[b:e] = x[b:e][::-1]
        is_[b:e] = i[b:e][::-1]
    m1 = engine.ParallelSparseMatrix(200, 60, xs, is_, p, True)
    m2 = engine.ParallelSparseMatrix(200, 60, x, i, p, True)
    v = np.random.default_rng(2).standard_normal(60)
    np.testing.assert_allclose(m1.multiply(v), m2.multiply(v), rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(m1.multiply(v), dense @ v, rtol=1e-12, atol=1e-12)
    bad = i.copy()
    bad[len(bad) // 2] = 200
    for on in (True, False):
        engine.set_device_ingest(on)
        try:
            with pytest.raises(engine.IrlbaError, match="index out of range"):
                engine.ParallelSparseMatrix(200, 60, x, bad, p, True)
        finally:
            engine.set_device_ingest(True)


@pytest.fixture
def tiny_staging(engine):
    """Stage every copy of 4 KiB or more through 4 KiB pinned slices (many
    slices per worker, both buffers of every lane in use)."""
    engine.set_staging(4096, 4096)
    try:
        yield
    finally:
        engine.set_staging(16 << 20, 8 << 20)


@pytest.mark.parametrize("device_ingest", [True, False])
def test_staged_copies_match_plain_copies(engine, tiny_staging, device_ingest):
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_pca_input(300, 9000, 0.1, seed=31, dtype=np.float32, cell_major=False)
    opts = engine.Options(seed=13)

    def run():
        engine.set_device_ingest(device_ingest)
        try:
            mat = engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major,
                                              form=engine.FORM_FP32_FP64STEPS)
        finally:
            engine.set_device_ingest(True)
        return mat, engine.pca(mat, True, True, 6, opts)

    staged_mat, staged = run()
    engine.set_staging(-1, 4096)
    plain_mat, plain = run()
    engine.set_staging(4096, 4096)
    assert staged.scores.nbytes > 16 * 4096
    np.testing.assert_array_equal(staged.scores, plain.scores)
    np.testing.assert_array_equal(staged.rotation, plain.rotation)
    np.testing.assert_array_equal(staged.variances, plain.variances)
    # Most copies end in a partial slice (nnz * 4 bytes is no multiple of 4 KiB).
    assert (inp.nnz * 4) % 4096 != 0
    _same_products(engine, staged_mat, plain_mat, inp.nrow, inp.ncol)
