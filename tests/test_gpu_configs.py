"""Parity at the workload shapes the benchmarks are quoted on, through the C ABI.

* Dense planted-rank 1000 x 200 (rank 10, singular values 100, 90, ..., 10 plus
  N(0, 1) noise), compute_simple k=5, extra_work=7, seeded start vector: the
  plain FP64 GPU path against the oracle (singular values 1e-10 relative,
  per-column sines 1e-8, identical restart count) and against LAPACK at the
  reference's own tolerance ladder (tests/src/compute.cpp:15-31, :92-123).
* Sparse 20,000 genes x 50,000 cells, ~5 % dense, FP64 values (CSC genes x
  cells, i.e. the cells x genes CSR pca input), centred and scaled pca k=50,
  tol 1e-5: plain FP64 GPU against the FP64 oracle at full size (singular
  vectors compared as the test's docstring explains).
* Sparse 2,000 genes x 200,000 cells, ~10 % dense, FP32 values (the 1.3M-cell
  headline matrix's shape, one sixth of its cells): the FP32+FP64-steps form
  against the FP64 oracle on the same (FP32-rounded) values, singular values
  within 1e-6 relative.
* dense == sparse CSC == sparse CSR pca results (tests/src/pca.cpp:218-240).
* The device restart step's update_k over the reference's 5^4 grid
  (tests/src/compute.cpp:52-76), bit-exact.
"""
import json
import os

import numpy as np
import pytest

from conftest import column_sines, principal_sines, same_same

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
THREADS = os.cpu_count() or 1


def test_update_k_device_matches_reference_grid(engine):
    kats = json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))["update_k"]
    quads = np.array([row[:4] for row in kats], dtype=np.int32)
    expected = np.array([row[4] for row in kats], dtype=np.int32)
    assert len(kats) == 625
    np.testing.assert_array_equal(engine.update_k_device(quads), expected)


def test_planted_dense_1000x200_k5(engine, oracle_mod):
    from cppirlba_gb300 import datagen
    A = datagen.dense_planted()           # 1000 x 200, rank 10 planted + N(0, 1)
    assert A.shape == (1000, 200)
    init = datagen.start_vector(200)
    opts = dict(initial=init, extra_work=7, exact_for_large_number=False)
    gpu = engine.compute_simple(A, 5, engine.Options(**opts))
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 5, oracle_mod.options(**opts))
    np.testing.assert_allclose(gpu.D, orc["D"], rtol=1e-10, atol=0)
    assert gpu.iterations == orc["iterations"] and gpu.converged == orc["converged"]
    assert np.max(column_sines(gpu.U, orc["U"])) < 1e-8
    assert np.max(column_sines(gpu.V, orc["V"])) < 1e-8

    # The reference's ladder against an exact SVD: tol 1e-9 gives singular
    # values and vectors within 1e-6 (compute.cpp:92-123, same_same).
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    tight = engine.compute_simple(A, 5, engine.Options(convergence_tolerance=1e-9, **opts))
    for j in range(5):
        assert same_same(tight.D[j], S[j], 1e-6)
    assert np.max(column_sines(tight.U, U[:, :5])) < 1e-6
    assert np.max(column_sines(tight.V, Vt[:5].T)) < 1e-6
    # The planted directions dominate: the top five singular values are the
    # planted 100, 90, ..., 60 lifted by the noise (about sqrt(s^2 + 1200)),
    # well above the noise bulk (about sqrt(1000) + sqrt(200) = 45.8).
    lifted = np.sqrt(np.array([100.0, 90, 80, 70, 60]) ** 2 + 1200)
    assert np.all(np.abs(gpu.D - lifted) < 3) and gpu.D[-1] > 50


def test_scrna_20k_x_50k_fp64_pca_full_size(engine, oracle_mod):
    """759 restarts to tol 1e-5 with neighbouring singular values as close as
    3.3e-5 relative. Two FP64 runs that differ only in rounding agree here in
    the way perturbation theory predicts (Davis-Kahan / Wedin): the sine between
    the two j-th singular vectors is about delta / gap_j, gap_j the relative gap
    to the nearest neighbouring singular value, with delta about 5e-13 between
    this engine and the oracle and 1e-13 between the oracle with the reference's
    two-sided Jacobi restart SVD and the oracle with a one-sided one. The 1e-8
    sine bound is therefore asserted on the principal angles between the
    subspaces and on every column with gap_j >= 1e-4, and as delta = sine x gap
    <= 1e-12 on every column (on the closer columns 1e-8 would need delta below
    3.3e-13, the spread of equally valid FP64 restart SVDs)."""
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_csc_20k()         # 20,000 genes x 50,000 cells, 5 %, FP64
    assert (inp.nrow, inp.ncol) == (50000, 20000) and inp.nnz > 45_000_000
    init = datagen.start_vector(inp.ncol)
    mat = engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major)
    gpu = engine.pca(mat, True, True, 50, engine.Options(initial=init))
    spec = oracle_mod.Spec.sparse(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major, THREADS)
    orc = oracle_mod.pca(spec, True, True, 50, oracle_mod.options(initial=init), dense_threads=THREADS)
    assert gpu.converged and orc["converged"]
    assert gpu.iterations == orc["iterations"]
    # variances = D^2 / (m - 1): 2e-10 on variances is 1e-10 on D.
    np.testing.assert_allclose(gpu.variances, orc["variances"], rtol=2e-10, atol=0)
    sv = np.sqrt(orc["variances"])
    rel = (sv[:-1] - sv[1:]) / sv[1:]
    gap = np.minimum(np.r_[np.inf, rel], np.r_[rel, np.inf])
    for a, b in ((gpu.rotation, orc["rotation"]), (gpu.scores, orc["scores"])):
        assert principal_sines(a, b).max() < 1e-8
        sines = column_sines(a, b)
        print("per-column sines: max %.2e; max sine x gap %.2e" % (sines.max(), (sines * gap).max()))
        assert np.all(sines[gap >= 1e-4] < 1e-8)
        assert np.all(sines * gap <= 1e-12)
    np.testing.assert_allclose(gpu.center, orc["center"], rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(gpu.scale, orc["scale"], rtol=1e-12)


def test_scrna_2k_x_200k_fp32_form_vs_fp64_oracle(engine, oracle_mod):
    """FP32 matrix, basis and matvecs with FP64 steps: singular values within
    1e-6 relative of the FP64 oracle on the same values; the subspaces agree to
    the FP32 basis's precision."""
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_pca_input(2000, 200000, 0.10, seed=3, dtype=np.float32, cell_major=False)
    assert inp.nnz > 38_000_000
    init = datagen.start_vector(inp.ncol)
    mat = engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major,
                                      form=engine.FORM_FP32_FP64STEPS)
    gpu = engine.pca(mat, True, True, 50, engine.Options(initial=init))
    spec = oracle_mod.Spec.sparse(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, inp.column_major, THREADS)
    orc = oracle_mod.pca(spec, True, True, 50, oracle_mod.options(initial=init), dense_threads=THREADS)
    assert gpu.converged and orc["converged"]
    m = inp.nrow
    D_gpu = np.sqrt(gpu.variances * (m - 1))
    D_orc = np.sqrt(orc["variances"] * (m - 1))
    rel = np.abs(D_gpu - D_orc) / D_orc
    print("FP32 form vs FP64 oracle: max rel D err %.3e, restarts %d vs %d, subspace sine %.2e" %
          (rel.max(), gpu.iterations, orc["iterations"], principal_sines(gpu.rotation, orc["rotation"]).max()))
    assert rel.max() <= 1e-6
    assert principal_sines(gpu.rotation, orc["rotation"]).max() < 1e-3
    assert np.max(column_sines(gpu.rotation[:, :10], orc["rotation"][:, :10])) < 1e-3


def test_pca_dense_equals_sparse_layouts(engine):
    # pca.cpp:218-240: dense == sparse == ParallelSparseMatrix at 1e-8.
    from cppirlba_gb300 import datagen
    inp = datagen.scrna_pca_input(300, 4000, 0.1, seed=29, dtype=np.float64, cell_major=False)
    dense = inp.to_dense()
    init = datagen.start_vector(inp.ncol)
    opts = engine.Options(initial=init)
    a = engine.pca(engine.SimpleMatrix(dense), True, True, 12, opts)
    b = engine.pca(engine.ParallelSparseMatrix(inp.nrow, inp.ncol, inp.val, inp.idx, inp.ptr, True), True, True, 12,
                   opts)
    csr = datagen.scrna_pca_input(300, 4000, 0.1, seed=29, dtype=np.float64, cell_major=True)
    c = engine.pca(engine.ParallelSparseMatrix(csr.nrow, csr.ncol, csr.val, csr.idx, csr.ptr, False), True, True, 12,
                   opts)
    for other in (b, c):
        for j in range(12):
            assert same_same(a.variances[j], other.variances[j], 1e-8)
        assert np.max(column_sines(a.rotation, other.rotation)) < 1e-8
        assert np.max(column_sines(a.scores, other.scores)) < 1e-8
