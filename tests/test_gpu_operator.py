"""User-defined matrices: the counterpart of a caller's own irlba::Matrix
subclass (Matrix/interface.hpp:141-223), whose products the caller supplies.

* OperatorMatrix: host products (numpy callables). The IRLBA loop runs on the
  device and each product copies its vectors to the host and back.
* DeviceOperatorMatrix: device products enqueued on the engine's stream, here a
  residual matrix R = A - X B^T (tests/cpp/residual_operator.cu: A an engine
  sparse matrix, the low-rank correction in that file's own kernels) and a
  product written with torch on the engine's stream.

Each is checked through the C ABI against the oracle on the realized matrix with
the same start vector: singular values to 1e-10 relative, the same restart
count and vectors to 1e-8 principal-angle sine in the FP64 form; in the FP32
form singular values within 1e-6 and vectors within 1e-3 principal-angle sine
of the FP64 oracle (the tolerances of the stored-matrix FP32 tests).
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import column_sines, normal_matrix, principal_sines, simulate_compressed_sparse

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _assert_fp64_parity(gpu, orc):
    np.testing.assert_allclose(gpu.D, orc["D"], rtol=1e-10)
    assert gpu.iterations == orc["iterations"]
    assert gpu.converged == orc["converged"]
    assert np.max(principal_sines(gpu.U, orc["U"])) < 1e-8
    assert np.max(principal_sines(gpu.V, orc["V"])) < 1e-8


def _host_operator(engine, A, form=0, calls=None):
    def mul(x):
        if calls is not None:
            calls["mul"] += 1
        return A @ x

    def adj(y):
        if calls is not None:
            calls["adj"] += 1
        return A.T @ y

    return engine.OperatorMatrix(A.shape[0], A.shape[1], mul, adj, form=form)


def test_host_operator_compute_matches_oracle(engine, oracle_mod):
    A = normal_matrix(300, 80, seed=5)
    calls = {"mul": 0, "adj": 0}
    op = _host_operator(engine, A, calls=calls)
    init = np.random.default_rng(6).standard_normal(80)
    gpu = engine.compute(op, 6, engine.Options(initial=init))
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 6, oracle_mod.options(initial=init))
    _assert_fp64_parity(gpu, orc)
    # One call of the caller's function per product the engine counts.
    assert calls["mul"] + calls["adj"] == gpu.stats["matvecs"]
    assert calls["mul"] > 0 and calls["adj"] > 0


@pytest.mark.parametrize("order", ["scale_outer", "center_outer"])
def test_decorated_host_operator_matches_oracle(engine, oracle_mod, order):
    """CenteredMatrix / ScaledMatrix over a user operator: the centring and
    scaling run on the device around the caller's products."""
    rng = np.random.default_rng(8)
    A = normal_matrix(200, 60, seed=9) + 2.0
    c = A.mean(axis=0)
    if order == "scale_outer":
        s = A.std(axis=0, ddof=1)
        op = _host_operator(engine, A)
        mat = engine.ScaledMatrix(engine.CenteredMatrix(op, c), s, True, True)
        spec = oracle_mod.Spec.dense(A, center=c, scale=s, scale_column=True, scale_divide=True, center_outer=False)
    else:
        s = rng.uniform(0.5, 2.0, 200)  # row scaling, multiplied
        op = _host_operator(engine, A)
        mat = engine.CenteredMatrix(engine.ScaledMatrix(op, s, False, False), c)
        spec = oracle_mod.Spec.dense(A, center=c, scale=s, scale_column=False, scale_divide=False, center_outer=True)
    init = rng.standard_normal(60)
    gpu = engine.compute(mat, 5, engine.Options(initial=init))
    orc = oracle_mod.compute(spec, 5, oracle_mod.options(initial=init))
    _assert_fp64_parity(gpu, orc)
    x = rng.standard_normal(60)
    np.testing.assert_allclose(mat.multiply(x), oracle_mod.multiply(spec, x), rtol=1e-12, atol=1e-12)
    y = rng.standard_normal(200)
    np.testing.assert_allclose(mat.adjoint_multiply(y), oracle_mod.adjoint_multiply(spec, y), rtol=1e-12,
                               atol=1e-12)


def test_host_operator_fp32_form_error_vs_fp64_oracle(engine, oracle_mod):
    A = normal_matrix(400, 100, seed=12)
    op = _host_operator(engine, A, form=engine.FORM_FP32_FP64STEPS)
    init = np.random.default_rng(13).standard_normal(100)
    gpu = engine.compute(op, 5, engine.Options(initial=init))
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 5, oracle_mod.options(initial=init))
    assert gpu.converged
    rel = np.max(np.abs(gpu.D - orc["D"]) / orc["D"])
    assert rel < 1e-6, rel
    assert np.max(column_sines(gpu.U, orc["U"])) < 1e-3


@pytest.mark.parametrize("shape", [(40, 5), (5, 40)])
def test_host_operator_exact_path_and_realize(engine, shape):
    """Small matrices take the exact SVD (compute.hpp:30-46, 164-170), which
    realizes the operator by products with unit vectors along its smaller side."""
    A = normal_matrix(*shape, seed=21)
    op = _host_operator(engine, A)
    np.testing.assert_array_equal(op.realize(), A)
    gpu = engine.compute(op, 2)
    np.testing.assert_allclose(gpu.D, np.linalg.svd(A, compute_uv=False)[:2], rtol=1e-10)
    assert gpu.iterations == 0 and gpu.converged


def test_operator_errors(engine):
    A = normal_matrix(50, 30, seed=2)

    def broken(_x):
        raise ValueError("the residual model is not fitted")

    op = engine.OperatorMatrix(50, 30, broken, lambda y: A.T @ y)
    with pytest.raises(engine.IrlbaError) as e:
        engine.compute(op, 3)
    assert "user-defined product failed" in str(e.value)
    assert isinstance(e.value.__cause__, ValueError)

    wrong = engine.OperatorMatrix(50, 30, lambda x: np.zeros(7), lambda y: A.T @ y)
    with pytest.raises(engine.IrlbaError):
        engine.compute(wrong, 3)

    good = _host_operator(engine, A)
    with pytest.raises(engine.IrlbaError) as e:
        engine.pca(good, True, True, 3)
    assert e.value.status == engine.ERROR_UNSUPPORTED
    # Still usable after the failures.
    np.testing.assert_allclose(good.multiply(np.ones(30)), A @ np.ones(30), rtol=1e-12)


# ---- device products -----------------------------------------------------------


class _ResidualC(ctypes.Structure):
    _fields_ = [("A", ctypes.c_void_p), ("m", ctypes.c_int64), ("n", ctypes.c_int64), ("r", ctypes.c_int64),
                ("X", ctypes.c_void_p), ("B", ctypes.c_void_p), ("t", ctypes.c_void_p), ("f32", ctypes.c_int32)]


@pytest.fixture(scope="module")
def residual_lib(engine, tmp_path_factory):
    libdir = os.path.dirname(engine.library_path())
    out = str(tmp_path_factory.mktemp("residual") / "libresidual_operator.so")
    subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "residual_operator.cu"), "-o", out, "-L", libdir,
                    "-lirlba_gb300", "-Xlinker", "-rpath," + libdir], check=True)
    return ctypes.CDLL(out)


def _residual_case(seed):
    m, n, r = 400, 120, 3
    dense, x, i, p = simulate_compressed_sparse(m, n, density=0.2, seed=seed)
    rng = np.random.default_rng(seed + 1)
    X = rng.standard_normal((m, r))
    B = rng.standard_normal((n, r)) * 0.5
    return m, n, r, dense, x, i, p, X, B


@pytest.mark.parametrize("form", [0, 1])
def test_residual_device_operator_matches_oracle(engine, oracle_mod, residual_lib, form):
    import torch
    m, n, r, dense, x, i, p, X, B = _residual_case(31)
    f32 = form == engine.FORM_FP32_FP64STEPS
    tdt = torch.float32 if f32 else torch.float64
    A = engine.ParallelSparseMatrix(m, n, x.astype(np.float32) if f32 else x, i, p, True, form=form)
    Xd = torch.tensor(np.asfortranarray(X).ravel(order="F"), dtype=tdt, device="cuda")
    Bd = torch.tensor(np.asfortranarray(B).ravel(order="F"), dtype=tdt, device="cuda")
    td = torch.zeros(r, dtype=tdt, device="cuda")
    torch.cuda.synchronize()
    st = _ResidualC(A.handle.value, m, n, r, Xd.data_ptr(), Bd.data_ptr(), td.data_ptr(), int(f32))
    fptr = ctypes.cast(residual_lib.residual_product, ctypes.c_void_p).value
    R = engine.DeviceOperatorMatrix(m, n, fptr, form=form, user=ctypes.addressof(st))
    def rounded(a):  # the values the FP32 form actually holds
        return a.astype(np.float32).astype(np.float64) if f32 else a

    Rd = rounded(dense) - rounded(X) @ rounded(B).T
    init = np.random.default_rng(32).standard_normal(n)
    gpu = engine.compute(R, 6, engine.Options(initial=init))
    orc = oracle_mod.compute(oracle_mod.Spec.dense(Rd), 6, oracle_mod.options(initial=init))
    if f32:
        assert gpu.converged
        rel = np.max(np.abs(gpu.D - orc["D"]) / orc["D"])
        assert rel < 1e-6, rel
        assert np.max(column_sines(gpu.V, orc["V"])) < 1e-3
    else:
        _assert_fp64_parity(gpu, orc)
        v = np.random.default_rng(33).standard_normal(n)
        np.testing.assert_allclose(R.multiply(v), Rd @ v, rtol=1e-12, atol=1e-11)
        w = np.random.default_rng(34).standard_normal(m)
        np.testing.assert_allclose(R.adjoint_multiply(w), Rd.T @ w, rtol=1e-12, atol=1e-11)
    del R, A, st


def test_centred_residual_device_operator_matches_oracle(engine, oracle_mod, residual_lib):
    """Centring fused after a device product (the elementwise epilogue)."""
    import torch
    m, n, r, dense, x, i, p, X, B = _residual_case(41)
    A = engine.ParallelSparseMatrix(m, n, x, i, p, True)
    Xd = torch.tensor(X.ravel(order="F"), dtype=torch.float64, device="cuda")
    Bd = torch.tensor(B.ravel(order="F"), dtype=torch.float64, device="cuda")
    td = torch.zeros(r, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = _ResidualC(A.handle.value, m, n, r, Xd.data_ptr(), Bd.data_ptr(), td.data_ptr(), 0)
    fptr = ctypes.cast(residual_lib.residual_product, ctypes.c_void_p).value
    R = engine.DeviceOperatorMatrix(m, n, fptr, user=ctypes.addressof(st))
    Rd = dense - X @ B.T
    c = Rd.mean(axis=0)
    s = Rd.std(axis=0, ddof=1)
    mat = engine.ScaledMatrix(engine.CenteredMatrix(R, c), s, True, True)
    spec = oracle_mod.Spec.dense(Rd, center=c, scale=s, scale_column=True, scale_divide=True, center_outer=False)
    init = np.random.default_rng(42).standard_normal(n)
    gpu = engine.compute(mat, 5, engine.Options(initial=init))
    orc = oracle_mod.compute(spec, 5, oracle_mod.options(initial=init))
    _assert_fp64_parity(gpu, orc)
    del mat, R, A, st


class _DeviceVector:
    """A device vector in the __cuda_array_interface__ protocol (for torch)."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (ptr, False), "version": 3,
                                         "strides": None}


def test_python_device_operator_with_torch_products(engine, oracle_mod):
    import torch
    A = normal_matrix(250, 70, seed=51)
    At = torch.tensor(A, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()

    def product(adjoint, xp, yp, stream):
        n_in, n_out = (250, 70) if adjoint else (70, 250)
        xv = torch.as_tensor(_DeviceVector(xp, n_in, "<f8"), device="cuda")
        yv = torch.as_tensor(_DeviceVector(yp, n_out, "<f8"), device="cuda")
        with torch.cuda.stream(torch.cuda.ExternalStream(stream)):
            yv.copy_((At.T if adjoint else At) @ xv)

    op = engine.DeviceOperatorMatrix(250, 70, product)
    init = np.random.default_rng(52).standard_normal(70)
    gpu = engine.compute(op, 5, engine.Options(initial=init))
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 5, oracle_mod.options(initial=init))
    # torch's GEMV sums in its own order: values to 1e-10, restarts identical.
    _assert_fp64_parity(gpu, orc)
