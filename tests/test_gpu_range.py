"""Argument ranges the reference accepts, through the C ABI: working subspaces
above 128 and above 1024 columns (compute.hpp:59-67,172: any number +
extra_work up to the smaller dimension) and exact SVDs of matrices whose
smaller dimension is above 1024 (compute.hpp:30-46,164-170)."""
import numpy as np
import pytest

from conftest import column_sines

pytestmark = pytest.mark.gpu


def planted(nr, nc, sv, seed):
    rng = np.random.default_rng(seed)
    U, _ = np.linalg.qr(rng.standard_normal((nr, len(sv))))
    V, _ = np.linalg.qr(rng.standard_normal((nc, len(sv))))
    return (U * sv) @ V.T


def test_working_subspace_above_128_matches_oracle(engine, oracle_mod):
    # number 130 + extra_work 10 = 140 columns: the wide rotation and the
    # one-CTA restart SVD, against the oracle at the usual FP64 tolerances.
    sv = 100.0 * 0.97 ** np.arange(300)
    A = planted(500, 300, sv, seed=31) + 1e-3 * np.random.default_rng(32).standard_normal((500, 300))
    init = np.random.default_rng(33).standard_normal(300)
    opts = dict(initial=init, extra_work=10)
    gpu = engine.compute(engine.SimpleMatrix(A), 130, engine.Options(**opts))
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 130, oracle_mod.options(**opts))
    assert gpu.converged == orc["converged"] and gpu.iterations == orc["iterations"]
    np.testing.assert_allclose(gpu.D, orc["D"], rtol=1e-10, atol=0)
    assert np.max(column_sines(gpu.U, orc["U"])) < 1e-8
    assert np.max(column_sines(gpu.V, orc["V"])) < 1e-8


def test_exact_svd_above_1024(engine):
    # number >= half the smaller dimension (1,100) selects the exact SVD.
    A = np.random.default_rng(41).standard_normal((1400, 1100))
    gpu = engine.compute(engine.SimpleMatrix(A), 600)
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    assert gpu.iterations == 0 and gpu.converged
    np.testing.assert_allclose(gpu.D, S[:600], rtol=1e-12, atol=1e-12 * S[0])
    # Singular vectors of a random matrix are well separated at the top.
    assert np.max(column_sines(gpu.U[:, :100], U[:, :100])) < 1e-8
    assert np.max(column_sines(gpu.V[:, :100], Vt[:100].T)) < 1e-8


def test_working_subspace_above_1024(engine):
    # Rank 1,040 with number 1,030 + extra_work 7 = 1,037 columns: the Lanczos
    # basis nearly spans the range, so the restarts converge quickly; the
    # restart SVD of B (1,037 x 1,037) goes through the large-matrix path.
    sv = np.linspace(50.0, 1.0, 1040)
    A = planted(2300, 2200, sv, seed=51)
    gpu = engine.compute(engine.SimpleMatrix(A), 1030, engine.Options(convergence_tolerance=1e-8))
    assert gpu.converged
    np.testing.assert_allclose(gpu.D, sv[:1030], rtol=1e-8)
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    rec = (gpu.U[:, :40] * gpu.D[:40]) @ gpu.V[:, :40].T
    np.testing.assert_allclose(rec, (U[:, :40] * S[:40]) @ Vt[:40], atol=1e-8 * S[0])
