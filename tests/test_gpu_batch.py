"""Batched form: many uneven PCAs in one persistent launch.

Each matrix of a batch must give what a separate irlba::pca call with the same
arguments gives (pca.hpp:55-139): checked against the FP64 oracle on the same
FP32-rounded input and start vector, at the FP32 form's tolerances: variances
within 2e-6 relative (singular values within 1e-6; measured up to 8e-8) and
rotation and score columns within principal-angle sines of 1e-3 (measured up
to 1.6e-5); and against the single-matrix FP32 form of the engine.
"""
import numpy as np
import pytest

from conftest import column_sines

pytestmark = pytest.mark.gpu

VAR_TOL = 2e-6
VEC_TOL = 1e-3


def _inputs(sizes, genes, density=0.08, seed=31, cell_major=False):
    from cppirlba_gb300 import datagen
    return datagen.scrna_batch(sizes, genes=genes, density=density, seed=seed, dtype=np.float32,
                               cell_major=cell_major)


def _batch(engine, inputs):
    cm = inputs[0].column_major
    return engine.Batch([(x.nrow, x.ncol, x.val, x.idx, x.ptr) for x in inputs], cm)


def _oracle(oracle_mod, x, center, scale, number, init, **kw):
    spec = oracle_mod.Spec.sparse(x.nrow, x.ncol, x.val.astype(np.float64), x.idx, x.ptr, x.column_major, 4)
    return oracle_mod.pca(spec, center, scale, number, oracle_mod.options(initial=init, **kw), dense_threads=4)


def _close(res, orc, var_tol=VAR_TOL, vec_tol=VEC_TOL):
    rel = np.max(np.abs(res.variances - orc["variances"]) / orc["variances"])
    assert rel < var_tol, rel
    assert np.max(column_sines(res.rotation, orc["rotation"])) < vec_tol
    assert np.max(column_sines(res.scores, orc["scores"])) < vec_tol


@pytest.mark.parametrize("center,scale", [(True, False), (True, True), (False, False), (False, True)])
def test_batch_matches_oracle(engine, oracle_mod, center, scale):
    sizes = [1500, 120, 800, 60, 2600, 300, 45, 1000]
    genes = 250
    inputs = _inputs(sizes, genes)
    init = np.random.default_rng(7).standard_normal(genes)
    b = _batch(engine, inputs)
    st = b.pca(center, scale, 6, engine.Options(initial=init))
    assert st["single"] == 0 and st["team"] in (1, 2, 4, 8) and st["ctas"] % st["team"] == 0
    for j, x in enumerate(inputs):
        res = b.result(j)
        assert res.stats["status"] == engine.BATCH_OK
        orc = _oracle(oracle_mod, x, center, scale, 6, init)
        assert res.converged == orc["converged"]
        _close(res, orc)
        if center:
            np.testing.assert_allclose(res.center, orc["center"], rtol=1e-12, atol=1e-15)
        if scale:
            np.testing.assert_allclose(res.scale, orc["scale"], rtol=1e-12)
    b.close()


@pytest.mark.parametrize("team,joint", [(1, -1), (2, 5), (4, 5), (4, 2), (4, 0), (8, 5), (8, 0)])
def test_batch_team_sizes(engine, oracle_mod, team, joint):
    """Every team size (CTAs per team, a thread-block cluster), with all, some
    or none of the matrices solved jointly, gives the oracle's results, down to
    matrices of a few dozen cells split over the team."""
    sizes = [3100, 40, 640, 25, 1800]
    genes = 180
    inputs = _inputs(sizes, genes, seed=47)
    init = np.random.default_rng(8).standard_normal(genes)
    b = _batch(engine, inputs)
    b.set_team(team, joint)
    st = b.pca(True, True, 3, engine.Options(initial=init))
    assert st["team"] == team and st["ctas"] % team == 0
    if team > 1:
        assert st["joint"] == joint
    for j, x in enumerate(inputs):
        res = b.result(j)
        orc = _oracle(oracle_mod, x, True, True, 3, init)
        if res.stats["status"] == engine.BATCH_OK:
            _close(res, orc)
        else:
            assert res.stats["status"] == engine.BATCH_SINGLE
            _close(res, orc, var_tol=1e-4)
    b.close()


def test_batch_matches_single_matrix_form(engine):
    sizes = [700, 2100, 90]
    genes = 400
    inputs = _inputs(sizes, genes, seed=37, cell_major=True)
    b = _batch(engine, inputs)
    opt = engine.Options(seed=99)
    b.pca(True, False, 8, opt)
    for j, x in enumerate(inputs):
        res = b.result(j)
        mat = engine.ParallelSparseMatrix(x.nrow, x.ncol, x.val, x.idx, x.ptr, x.column_major,
                                          form=engine.FORM_FP32_FP64STEPS)
        one = engine.pca(mat, True, False, 8, opt)
        rel = np.max(np.abs(res.variances - one.variances) / one.variances)
        assert rel < VAR_TOL
        assert np.max(column_sines(res.rotation, one.rotation)) < VEC_TOL
    b.close()


def test_batch_repeat_is_deterministic_and_reuses_graph(engine):
    inputs = _inputs([500, 1300, 75, 900], 300, seed=41)
    b = _batch(engine, inputs)
    st1 = b.pca(True, True, 5)
    r1 = [b.result(j) for j in range(len(inputs))]
    st2 = b.pca(True, True, 5)
    r2 = [b.result(j) for j in range(len(inputs))]
    assert st1["graph_captured"] == 1 and st2["graph_captured"] == 0
    assert st2["tune_ms"] == 0.0
    for a, c in zip(r1, r2):
        np.testing.assert_array_equal(a.variances, c.variances)
        np.testing.assert_array_equal(a.rotation, c.rotation)
        np.testing.assert_array_equal(a.scores, c.scores)
    st3 = b.pca(True, True, 4)
    assert st3["graph_captured"] == 1
    b.close()


def test_batch_tuned_and_fixed_groups(engine, oracle_mod):
    sizes = [3000, 150, 1200]
    genes = 600
    inputs = _inputs(sizes, genes, seed=43)
    init = np.random.default_rng(3).standard_normal(genes)
    b = _batch(engine, inputs)
    b.pca(True, False, 5, engine.Options(initial=init))
    gm, ga = b.groups()
    assert set(gm.tolist()) <= {4, 8, 16, 32} and set(ga.tolist()) <= {4, 8, 16, 32}
    orcs = [_oracle(oracle_mod, x, True, False, 5, init) for x in inputs]
    for g in (4, 32):
        b.set_groups(np.full(len(sizes), g), np.full(len(sizes), g))
        st = b.pca(True, False, 5, engine.Options(initial=init))
        assert st["tune_ms"] == 0.0
        for j in range(len(sizes)):
            res = b.result(j)
            assert res.stats["group_mul"] == g and res.stats["group_adj"] == g
            _close(res, orcs[j])
    b.close()


def test_batch_unstaged_and_single_matrix_paths(engine, oracle_mod):
    """Observations beyond the shared-memory stage (global gathers), a matrix
    that needs the exact SVD, and an all-zero matrix whose start vector lies
    in the null space (compute.hpp:30-46, lanczos.hpp:79-82)."""
    from cppirlba_gb300 import datagen
    big = datagen.scrna_pca_input(60, 56000, 0.05, 51, np.float32, False)
    small = datagen.scrna_pca_input(5, 300, 0.5, 52, np.float32, False)
    mid = datagen.scrna_pca_input(60, 900, 0.1, 53, np.float32, False)
    zp = np.zeros(61, dtype=np.int64)
    zero = datagen.SparseInput(400, 60, zp, np.zeros(0, dtype=np.int32), np.zeros(0, dtype=np.float32),
                               column_major=True)
    inputs = [big, small, mid, zero]
    b = engine.Batch([(x.nrow, x.ncol, x.val, x.idx, x.ptr) for x in inputs], True)
    opt = engine.Options(seed=5)
    st = b.pca(True, False, 3, opt)
    assert st["single"] == 2
    infos = [b.result(j).stats for j in range(4)]
    assert infos[0]["status"] == engine.BATCH_OK and infos[2]["status"] == engine.BATCH_OK
    assert infos[1]["status"] == engine.BATCH_SINGLE
    assert infos[3]["status"] == engine.BATCH_FAILED and infos[3]["error"] == engine.ERROR_NUMERICAL
    for j in (0, 1, 2):
        x = inputs[j]
        spec = oracle_mod.Spec.sparse(x.nrow, x.ncol, x.val.astype(np.float64), x.idx, x.ptr, True, 4)
        orc = oracle_mod.pca(spec, True, False, 3, oracle_mod.options(seed=5), dense_threads=4)
        _close(b.result(j), orc)
    b.close()


def test_batch_argument_errors(engine):
    inputs = _inputs([100, 200], 50, seed=61)
    b = _batch(engine, inputs)
    with pytest.raises(engine.IrlbaError, match="cannot be greater"):
        b.pca(True, False, 60)
    with pytest.raises(engine.IrlbaError, match="index out of range"):
        b.result(5)
    b.close()
    with pytest.raises(engine.IrlbaError, match="matrix 1"):
        engine.Batch([(3, 3, np.ones(1), np.array([0]), np.array([0, 1, 1, 1])),
                      (3, 3, np.ones(1), np.array([7]), np.array([0, 1, 1, 1]))], True)
    empty = engine.Batch([], True)
    st = empty.pca(True, False, 2)
    assert st["ctas"] == 0
    empty.close()
