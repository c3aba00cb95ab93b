"""GPU IRLBA parity through the C ABI against the oracle (CppIrlba's
compute.hpp / pca.hpp restated on the CPU).

Plain FP64 form: singular values within 1e-10 relative, U and V within 1e-8 in
principal-angle sine (per column, sign-agnostic), identical restart counts and
convergence flags, same inputs and start vector. FP32+FP64-steps form: the
error against the FP64 oracle is measured and bounded per test."""
import numpy as np
import pytest

from conftest import column_sines, normal_matrix, same_same, simulate_compressed_sparse, to_csr

pytestmark = pytest.mark.gpu

D_TOL = 1e-10
VEC_TOL = 1e-8


def _check(gpu, orc, d_tol=D_TOL, vec_tol=VEC_TOL, same_iters=True):
    assert gpu.D.shape == orc["D"].shape
    np.testing.assert_allclose(gpu.D, orc["D"], rtol=d_tol, atol=d_tol * max(orc["D"].max(), 1e-300))
    if same_iters:
        assert gpu.iterations == orc["iterations"]
        assert gpu.converged == orc["converged"]
    nz = orc["D"] > 1e-8 * max(orc["D"].max(), 1e-300)
    if nz.any():
        assert np.max(column_sines(gpu.U[:, nz], orc["U"][:, nz])) < vec_tol
        assert np.max(column_sines(gpu.V[:, nz], orc["V"][:, nz])) < vec_tol


def _opts(engine, oracle_mod, **kw):
    return engine.Options(**kw), oracle_mod.options(**kw)


@pytest.mark.parametrize("nr,nc,rank", [(20, 10, 5), (100, 50, 5), (50, 100, 10), (300, 200, 8), (200, 300, 3)])
def test_dense_compute_parity(engine, oracle_mod, nr, nc, rank):
    A = normal_matrix(nr, nc)
    init = np.random.default_rng(7).standard_normal(nc)
    go, oo = _opts(engine, oracle_mod, initial=init, exact_for_large_number=False)
    gpu = engine.compute(engine.SimpleMatrix(A), rank, go)
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), rank, oo)
    _check(gpu, orc)
    # and vs LAPACK at the reference's test tolerances (compute.cpp:15-31, 92-123)
    S = np.linalg.svd(A, compute_uv=False)
    np.testing.assert_allclose(gpu.D, S[:rank], rtol=1e-4)


def test_default_start_vector_matches_oracle(engine, oracle_mod):
    # No `initial`: both draw Box-Muller normals from std::mt19937_64(seed).
    A = normal_matrix(120, 80, seed=3)
    for seed in (5489, 1234):
        gpu = engine.compute(engine.SimpleMatrix(A), 6, engine.Options(seed=seed))
        orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 6, oracle_mod.options(seed=seed))
        _check(gpu, orc)


def test_compute_tight_tolerance_matches_lapack(engine):
    A = normal_matrix(100, 50, seed=11)
    gpu = engine.compute(engine.SimpleMatrix(A), 10, engine.Options(convergence_tolerance=1e-9))
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    np.testing.assert_allclose(gpu.D, S[:10], rtol=1e-6)
    assert np.max(column_sines(gpu.U, U[:, :10])) < 1e-5
    assert np.max(column_sines(gpu.V, Vt[:10].T)) < 1e-5


@pytest.mark.parametrize("column_major", [True, False])
@pytest.mark.parametrize("nr,nc,rank", [(99, 64, 5), (400, 250, 12), (2000, 900, 20)])
def test_sparse_compute_parity(engine, oracle_mod, nr, nc, rank, column_major):
    dense, x, i, p = simulate_compressed_sparse(nr, nc, density=0.2 if nr < 1000 else 0.05)
    init = np.random.default_rng(8).standard_normal(nc)
    go, oo = _opts(engine, oracle_mod, initial=init)
    if column_major:
        mat = engine.ParallelSparseMatrix(nr, nc, x, i, p, True)
        spec = oracle_mod.Spec.sparse(nr, nc, x, i, p, True)
    else:
        xr, ir, pr = to_csr(dense)
        mat = engine.ParallelSparseMatrix(nr, nc, xr, ir, pr, False)
        spec = oracle_mod.Spec.sparse(nr, nc, xr, ir, pr, False)
    _check(engine.compute(mat, rank, go), oracle_mod.compute(spec, rank, oo))


def test_dense_equals_sparse(engine):
    # compute.cpp:240-271: dense == sparse == ParallelSparseMatrix
    dense, x, i, p = simulate_compressed_sparse(99, 64)
    go = engine.Options(extra_work=7)
    a = engine.compute(engine.SimpleMatrix(dense), 8, go)
    b = engine.compute(engine.ParallelSparseMatrix(99, 64, x, i, p, True), 8, go)
    np.testing.assert_allclose(a.D, b.D, rtol=1e-8)
    assert np.max(column_sines(a.U, b.U)) < 1e-7
    assert np.max(column_sines(a.V, b.V)) < 1e-7


def test_max_iterations_quirk(engine, oracle_mod):
    # Not converged: outputs combine the rotated bases with the previous SVD of B
    # (compute.hpp:268-280 then :302-305), as the reference does.
    A = normal_matrix(300, 200, seed=21)
    init = np.random.default_rng(2).standard_normal(200)
    go, oo = _opts(engine, oracle_mod, initial=init, max_iterations=3, convergence_tolerance=1e-12)
    gpu = engine.compute(engine.SimpleMatrix(A), 10, go)
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 10, oo)
    assert not gpu.converged and gpu.iterations == 3
    _check(gpu, orc)


@pytest.mark.parametrize("shape,number,opts", [((10, 3), 2, {}), ((20, 50), 15, {}), ((20, 50), 20, {}),
                                               ((20, 50), 50, {"cap_number": True}), ((50, 4), 2, {})])
def test_exact_fallback(engine, shape, number, opts):
    A = normal_matrix(*shape, seed=sum(shape))
    gpu = engine.compute(engine.SimpleMatrix(A), number, engine.Options(**opts))
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    r = min(number, min(shape))
    assert gpu.iterations == 0 and gpu.converged
    np.testing.assert_allclose(gpu.D, S[:r], rtol=1e-12, atol=1e-12 * S[0])
    assert np.max(column_sines(gpu.U, U[:, :r])) < 1e-8
    assert np.max(column_sines(gpu.V, Vt[:r].T)) < 1e-8


def test_errors(engine):
    # compute.cpp:193-238 message substrings
    m = engine.SimpleMatrix(normal_matrix(20, 10))
    with pytest.raises(engine.IrlbaError, match="cannot be greater than"):
        engine.compute(m, 100)
    with pytest.raises(engine.IrlbaError, match="must be less than"):
        engine.compute(m, 10, engine.Options(exact_for_large_number=False))
    with pytest.raises(engine.IrlbaError, match="must be positive"):
        engine.compute(m, 0, engine.Options(extra_work=0))
    with pytest.raises(engine.IrlbaError, match="^initialization"):
        engine.compute(m, 2, engine.Options(initial=np.zeros(1)))
    with pytest.raises(engine.IrlbaError, match="null space"):
        engine.compute(engine.SimpleMatrix(np.zeros((30, 20))), 3)


@pytest.mark.parametrize("rank", [2, 5, 10])
def test_invariant_subspace_refill(engine, oracle_mod, rank):
    # invariant.cpp:7-86: exact low rank forces the random refill of
    # lanczos.hpp:101-106,124-129 (the careful restart path on the GPU).
    rng = np.random.default_rng(42)
    A = np.zeros((100, 50))
    A[:, :rank] = rng.standard_normal((100, rank))
    for c in range(rank, 50):
        A[:, c] = A[:, c % rank]
    gpu = engine.compute(engine.SimpleMatrix(A), rank + 3)
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), rank + 3)
    assert np.all(gpu.D[:rank] > 0.01) and np.all(gpu.D[rank:] < 1e-8)
    np.testing.assert_allclose(gpu.D[:rank], orc["D"][:rank], rtol=1e-10)
    assert gpu.stats["careful_restarts"] >= 1
    g2 = engine.compute(engine.SimpleMatrix(A), rank + 2)
    rec = g2.U @ np.diag(g2.D) @ g2.V.T
    np.testing.assert_allclose(rec, A, atol=1e-8 * np.abs(A).max())


def _spawn(A):
    mean = A.mean(axis=0)
    centered = A - mean
    both = centered / np.sqrt((centered ** 2).sum(axis=0) / (A.shape[0] - 1))
    scaled = A / np.sqrt((A ** 2).sum(axis=0) / (A.shape[0] - 1))
    return centered, scaled, both


@pytest.mark.parametrize("nr,nc,rank", [(100, 50, 5), (50, 100, 10), (300, 120, 8)])
def test_pca_parity(engine, oracle_mod, nr, nc, rank):
    A = normal_matrix(nr, nc)
    init = np.random.default_rng(5).standard_normal(nc)
    for center, scale in ((True, True), (True, False), (False, True), (False, False)):
        gpu = engine.pca(engine.SimpleMatrix(A), center, scale, rank, engine.Options(initial=init))
        orc = oracle_mod.pca(oracle_mod.Spec.dense(A), center, scale, rank, oracle_mod.options(initial=init))
        np.testing.assert_allclose(gpu.variances, orc["variances"], rtol=2e-10)
        assert gpu.iterations == orc["iterations"]
        assert np.max(column_sines(gpu.rotation, orc["rotation"])) < VEC_TOL
        assert np.max(column_sines(gpu.scores, orc["scores"])) < VEC_TOL
        if center:
            np.testing.assert_allclose(gpu.center, orc["center"], rtol=1e-13, atol=1e-15)
            for j in range(rank):
                assert abs(gpu.scores[:, j].sum()) < 1e-8
                assert same_same(np.sum(gpu.scores[:, j] ** 2) / (nr - 1), gpu.variances[j], 1e-8)
        if scale:
            np.testing.assert_allclose(gpu.scale, orc["scale"], rtol=1e-12)


def test_pca_sparse_scrna(engine, oracle_mod):
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_pca_input(300, 6000, 0.1, seed=17, dtype=np.float64, cell_major=False)
    init = datagen.start_vector(inp.ncol)
    mat = engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major)
    gpu = engine.pca(mat, True, True, 20, engine.Options(initial=init))
    spec = oracle_mod.Spec.sparse(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major, 4)
    orc = oracle_mod.pca(spec, True, True, 20, oracle_mod.options(initial=init), dense_threads=4)
    assert gpu.iterations == orc["iterations"] and gpu.converged == orc["converged"]
    np.testing.assert_allclose(gpu.variances, orc["variances"], rtol=2e-10)
    assert np.max(column_sines(gpu.rotation, orc["rotation"])) < VEC_TOL


def test_pca_errors(engine):
    with pytest.raises(engine.IrlbaError, match="cannot center"):
        engine.pca(engine.SimpleMatrix(np.zeros((0, 10))), True, True, 1)
    with pytest.raises(engine.IrlbaError, match="cannot scale"):
        engine.pca(engine.SimpleMatrix(normal_matrix(1, 10)), True, True, 1)
    out = engine.pca(engine.SimpleMatrix(np.zeros((10, 2))), True, True, 1)
    assert out.converged and np.all(np.isfinite(out.scores)) and np.all(np.isfinite(out.rotation))


def test_fp32_form_error_vs_fp64_oracle(engine, oracle_mod):
    """FP32 matrix/basis/matvecs, FP64 steps: singular values within 1e-6
    (variances within 2e-6) and rotation columns within principal-angle sines of
    1e-3 of the FP64 oracle on the same (FP32-rounded) input."""
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_pca_input(400, 20000, 0.1, seed=19, dtype=np.float32, cell_major=False)
    init = datagen.start_vector(inp.ncol)
    mat = engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major,
                                      form=engine.FORM_FP32_FP64STEPS)
    gpu = engine.pca(mat, True, True, 10, engine.Options(initial=init))
    spec = oracle_mod.Spec.sparse(inp.nrow, inp.ncol, inp.val.astype(np.float64), inp.idx, inp.ptr,
                                  inp.column_major, 4)
    orc = oracle_mod.pca(spec, True, True, 10, oracle_mod.options(initial=init), dense_threads=4)
    assert gpu.converged
    rel = np.max(np.abs(gpu.variances - orc["variances"]) / orc["variances"])
    assert rel < 2e-6
    assert np.max(column_sines(gpu.rotation, orc["rotation"])) < 1e-3


def test_fp64_runs_are_bit_reproducible(engine):
    dense, x, i, p = simulate_compressed_sparse(500, 300, seed=3)
    mat = engine.ParallelSparseMatrix(500, 300, x, i, p, True)
    a = engine.compute(mat, 10)
    b = engine.compute(mat, 10)
    np.testing.assert_array_equal(a.D, b.D)
    np.testing.assert_array_equal(a.U, b.U)
