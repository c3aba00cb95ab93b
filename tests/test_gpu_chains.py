"""Decorator chains beyond one CenteredMatrix and one ScaledMatrix (the
reference's decorators wrap any Matrix: centered.hpp:139-160,
scaled.hpp:195-223), through the C ABI, against the oracle on the realized
matrix: singular values 1e-10, vectors 1e-8, identical restart counts."""
import numpy as np
import pytest

from conftest import column_sines, simulate_compressed_sparse

pytestmark = pytest.mark.gpu


def realize(A, chain):
    """chain: decorators from the innermost out, as ("center", c) or
    ("scale", s, column, divide)."""
    M = A.copy()
    for d in chain:
        if d[0] == "center":
            M = M - d[1][None, :]
        else:
            s, column, divide = d[1], d[2], d[3]
            f = 1.0 / s if divide else s
            M = M * f[None, :] if column else M * f[:, None]
    return M


def build(engine, base, chain):
    m = base
    for d in chain:
        m = engine.CenteredMatrix(m, d[1]) if d[0] == "center" else engine.ScaledMatrix(m, d[1], d[2], d[3])
    return m


CHAINS = [
    "center/scale_row/center",
    "scale_col/scale_row",
    "center/center",
    "scale_row/center/scale_col/center",
]


@pytest.mark.parametrize("name", CHAINS)
@pytest.mark.parametrize("fp32", [False, True])
def test_nested_chain_matches_oracle(engine, oracle_mod, name, fp32):
    nr, nc = 300, 120
    dense, x, i, p = simulate_compressed_sparse(nr, nc, density=0.3, seed=61)
    rng = np.random.default_rng(62)
    parts = {
        "center": lambda: ("center", rng.standard_normal(nc) * 0.3),
        "scale_row": lambda: ("scale", rng.uniform(0.5, 2.0, nr), False, False),
        "scale_col": lambda: ("scale", rng.uniform(0.5, 2.0, nc), True, True),
    }
    chain = [parts[k]() for k in name.split("/")]
    form = engine.FORM_FP32_FP64STEPS if fp32 else engine.FORM_FP64
    xv = x.astype(np.float32).astype(np.float64) if fp32 else x
    base = engine.ParallelSparseMatrix(nr, nc, xv, i, p, True, form=form)
    dense = np.zeros((nr, nc))
    for c in range(nc):
        dense[i[p[c]:p[c + 1]], c] = xv[p[c]:p[c + 1]]
    M = realize(dense, chain)
    init = rng.standard_normal(nc)
    gpu = engine.compute(build(engine, base, chain), 8, engine.Options(initial=init))
    orc = oracle_mod.compute(oracle_mod.Spec.dense(M), 8, oracle_mod.options(initial=init))
    if fp32:
        # FP32 basis and products: singular values to the FP32 form's accuracy.
        np.testing.assert_allclose(gpu.D, orc["D"], rtol=1e-5)
        assert np.max(column_sines(gpu.V, orc["V"])) < 1e-3
    else:
        np.testing.assert_allclose(gpu.D, orc["D"], rtol=1e-10)
        assert gpu.iterations == orc["iterations"]
        assert np.max(column_sines(gpu.U, orc["U"])) < 1e-8
        assert np.max(column_sines(gpu.V, orc["V"])) < 1e-8
    # The chain's products through the plug-in surface (Workspace::multiply).
    mat = build(engine, base, chain)
    v = rng.standard_normal(nc)
    w = rng.standard_normal(nr)
    tol = 1e-5 if fp32 else 1e-12
    np.testing.assert_allclose(mat.multiply(v), M @ v, rtol=tol, atol=tol * np.abs(M @ v).max())
    np.testing.assert_allclose(mat.adjoint_multiply(w), M.T @ w, rtol=tol, atol=tol * np.abs(M.T @ w).max())
