"""GPU matvec parity through the C ABI: ParallelSparseMatrix / SimpleMatrix
multiply, adjoint multiply and realize, with every CenteredMatrix /
ScaledMatrix arrangement the engine fuses, against the oracle.
Tolerance: FP64 form 1e-12 relative (summation order differs); FP32 form 1e-5."""
import numpy as np
import pytest

from conftest import simulate_compressed_sparse, to_csr

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


SHAPES = [(10, 10), (49, 51), (97, 88), (1, 30), (30, 1), (300, 20000), (20000, 300)]


@pytest.mark.parametrize("nr,nc", SHAPES)
@pytest.mark.parametrize("column_major", [True, False])
def test_sparse_multiply(engine, oracle_mod, nr, nc, column_major):
    density = 0.2 if nr * nc < 1e6 else 0.01
    dense, x, i, p = simulate_compressed_sparse(nr, nc, density=density, seed=nr * 7 + nc)
    if column_major:
        mat = engine.ParallelSparseMatrix(nr, nc, x, i, p, True)
        spec = oracle_mod.Spec.sparse(nr, nc, x, i, p, True)
    else:
        xr, ir, pr = to_csr(dense)
        mat = engine.ParallelSparseMatrix(nr, nc, xr, ir, pr, False)
        spec = oracle_mod.Spec.sparse(nr, nc, xr, ir, pr, False)
    rng = np.random.default_rng(3)
    v = rng.standard_normal(nc)
    w = rng.standard_normal(nr)
    ref = oracle_mod.multiply(spec, v)
    out = np.full(nr, 123.0)  # dirty output must be overwritten
    mat.multiply(v, out)
    assert _rel(out, ref) < 1e-12
    mat.multiply(v, out)
    assert _rel(out, ref) < 1e-12
    ref2 = oracle_mod.adjoint_multiply(spec, w)
    out2 = np.full(nc, -7.0)
    mat.adjoint_multiply(w, out2)
    assert _rel(out2, ref2) < 1e-12
    np.testing.assert_array_equal(mat.realize(), dense)


def test_empty_rows_and_columns(engine, oracle_mod):
    dense = np.zeros((40, 30))
    dense[3, 5] = 2.0
    dense[39, 29] = -1.5
    dense[10, :] = 1.0
    x, i, p = to_csr(dense)
    mat = engine.ParallelSparseMatrix(40, 30, x, i, p, False)
    v = np.arange(30.0)
    np.testing.assert_allclose(mat.multiply(v), dense @ v, rtol=1e-14)
    w = np.arange(40.0)
    np.testing.assert_allclose(mat.adjoint_multiply(w), dense.T @ w, rtol=1e-14)
    z = engine.ParallelSparseMatrix(5, 4, np.zeros(0), np.zeros(0, np.int32), np.zeros(6, np.int64), False)
    np.testing.assert_array_equal(z.multiply(np.ones(4)), np.zeros(5))


@pytest.mark.parametrize("kind", ["dense_col", "dense_row", "sparse"])
@pytest.mark.parametrize("chain", ["center", "scale_col_div", "scale_row_mul", "scale_col(center)",
                                   "center(scale_col)", "scale_row_div(center)", "center(scale_row_mul)"])
def test_decorator_chains(engine, oracle_mod, kind, chain):
    nr, nc = 37, 23
    dense, x, i, p = simulate_compressed_sparse(nr, nc, seed=5)
    rng = np.random.default_rng(9)
    center = rng.standard_normal(nc)
    scol = rng.uniform(0.5, 2.0, nc)
    srow = rng.uniform(0.5, 2.0, nr)
    if kind == "sparse":
        base = engine.ParallelSparseMatrix(nr, nc, x, i, p, True)
    elif kind == "dense_col":
        base = engine.SimpleMatrix(np.asfortranarray(dense))
    else:
        base = engine.SimpleMatrix(np.ascontiguousarray(dense))
    args = dict(center=None, scale=None, scale_column=True, scale_divide=True, center_outer=False)
    if chain == "center":
        m = engine.CenteredMatrix(base, center)
        args.update(center=center)
    elif chain == "scale_col_div":
        m = engine.ScaledMatrix(base, scol, True, True)
        args.update(scale=scol)
    elif chain == "scale_row_mul":
        m = engine.ScaledMatrix(base, srow, False, False)
        args.update(scale=srow, scale_column=False, scale_divide=False)
    elif chain == "scale_col(center)":
        m = engine.ScaledMatrix(engine.CenteredMatrix(base, center), scol, True, True)
        args.update(center=center, scale=scol)
    elif chain == "center(scale_col)":
        m = engine.CenteredMatrix(engine.ScaledMatrix(base, scol, True, False), center)
        args.update(center=center, scale=scol, scale_divide=False, center_outer=True)
    elif chain == "scale_row_div(center)":
        m = engine.ScaledMatrix(engine.CenteredMatrix(base, center), srow, False, True)
        args.update(center=center, scale=srow, scale_column=False)
    else:
        m = engine.CenteredMatrix(engine.ScaledMatrix(base, srow, False, False), center)
        args.update(center=center, scale=srow, scale_column=False, scale_divide=False, center_outer=True)
    spec = oracle_mod.Spec.dense(dense, **args)
    v = rng.standard_normal(nc)
    w = rng.standard_normal(nr)
    assert _rel(m.multiply(v), oracle_mod.multiply(spec, v)) < 1e-12
    assert _rel(m.adjoint_multiply(w), oracle_mod.adjoint_multiply(spec, w)) < 1e-12
    np.testing.assert_allclose(m.realize(), oracle_mod.realize(spec), rtol=1e-14, atol=1e-14)


def test_double_centering_chain(engine):
    # A CenteredMatrix over a CenteredMatrix (the reference's decorators nest
    # freely) runs as a chain operator: M = I - 1 c1^T - 1 c2^T.
    base = engine.SimpleMatrix(np.eye(6))
    c1, c2 = np.arange(6.0), np.ones(6)
    m = engine.CenteredMatrix(engine.CenteredMatrix(base, c1), c2)
    M = np.eye(6) - c1[None, :] - c2[None, :]
    v = np.linspace(-1, 2, 6)
    np.testing.assert_allclose(m.multiply(v), M @ v, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(m.adjoint_multiply(v), M.T @ v, rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(m.realize(), M, rtol=1e-13, atol=1e-13)


def test_fp32_form_matvec(engine, oracle_mod):
    nr, nc = 500, 300
    dense, x, i, p = simulate_compressed_sparse(nr, nc, seed=77)
    m = engine.ParallelSparseMatrix(nr, nc, x.astype(np.float32), i, p, True, form=engine.FORM_FP32_FP64STEPS)
    d32 = dense.astype(np.float32).astype(np.float64)
    v = np.random.default_rng(1).standard_normal(nc)
    assert _rel(m.multiply(v), d32 @ v) < 1e-5
    w = np.random.default_rng(2).standard_normal(nr)
    assert _rel(m.adjoint_multiply(w), d32.T @ w) < 1e-5


def test_orthogonalize_vector_device(engine, oracle_mod):
    import torch
    rng = np.random.default_rng(4)
    L, c = 10000, 37
    Q, _ = np.linalg.qr(rng.standard_normal((L, c)))
    v = rng.standard_normal(L)
    ref = oracle_mod.orthogonalize_vector(Q, v, 25)
    Qd = torch.tensor(np.asfortranarray(Q).T.copy(), device="cuda")  # column j contiguous
    vd = torch.tensor(v, device="cuda")
    lib = engine.load_library()
    st = lib.irlba_gb300_orthogonalize_vector_device(Qd.data_ptr(), L, L, 25, vd.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(vd.cpu().numpy(), ref, rtol=1e-10, atol=1e-13)
