"""The header-style C++ drop-in (include/irlba_gb300/irlba.hpp), used the way a
CppIrlba caller uses irlba::compute / compute_simple / pca and the Matrix
decorators, checked against the oracle. The test program is compiled with g++
against the engine library at test time."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def dropin_output(engine, tmp_path_factory):
    libdir = os.path.dirname(engine.library_path())
    exe = str(tmp_path_factory.mktemp("dropin") / "dropin_test")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "dropin_test.cpp"), "-o", exe, "-L", libdir,
                    "-lirlba_gb300", "-Wl,-rpath," + libdir], check=True)
    out = subprocess.run([exe], check=True, stdout=subprocess.PIPE, text=True).stdout
    return json.loads(out)


def test_dropin_compute(dropin_output, oracle_mod):
    d = dropin_output
    nr, nc = 120, 70
    A = np.array(d["A_colmajor"]).reshape(nc, nr).T
    init = np.array(d["init"])
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 6, oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["compute_D"], orc["D"], rtol=1e-10)
    np.testing.assert_allclose(d["compute_simple_D"], orc["D"], rtol=1e-10)
    assert d["compute_iterations"] == orc["iterations"]
    u0 = np.array(d["compute_U0"])
    assert abs(abs(u0 @ orc["U"][:, 0]) - 1.0) < 1e-10
    p = oracle_mod.pca(oracle_mod.Spec.dense(A), True, True, 5, oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["pca_variances"], p["variances"], rtol=1e-10)
    assert d["pca_iterations"] == p["iterations"]


def test_dropin_decorated_sparse(dropin_output, oracle_mod):
    d = dropin_output
    nr, nc = 120, 70
    x, i, p = np.array(d["sparse_x"]), np.array(d["sparse_i"], dtype=np.int32), np.array(d["sparse_p"], dtype=np.int64)
    spec = oracle_mod.Spec.sparse(nr, nc, x, i, p, True, 1, center=np.array(d["center"]), scale=np.array(d["scale"]))
    init = np.array(d["init"])
    orc = oracle_mod.compute(spec, 4, oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["chain_D"], orc["D"], rtol=1e-10)
    assert d["chain_iterations"] == orc["iterations"]
    # The centre and scale vectors changed after the decorators were built:
    # the next compute uses the new contents (the reference reads them through
    # its pointers, centered.hpp:46-52, scaled.hpp:52-69). The workspace
    # multiply below ran after the vectors were restored.
    spec2 = oracle_mod.Spec.sparse(nr, nc, x, i, p, True, 1, center=np.array(d["center_changed"]),
                                   scale=np.array(d["scale_changed"]))
    orc2 = oracle_mod.compute(spec2, 4, oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["chain_changed_D"], orc2["D"], rtol=1e-10)
    assert d["chain_changed_iterations"] == orc2["iterations"]
    assert np.max(np.abs(np.array(d["chain_changed_D"]) - orc["D"]) / orc["D"]) > 1e-3
    np.testing.assert_allclose(d["chain_multiply_init"], oracle_mod.multiply(spec, init), rtol=1e-12, atol=1e-12)
    assert "cannot be greater than" in d["error_message"]


def test_dropin_strided_dense(dropin_output, oracle_mod):
    """A dense view with an outer stride (an Eigen Map with OuterStride, a
    Block): the engine reads the view's elements, not a contiguous prefix."""
    d = dropin_output
    nr, nc = 120, 70
    A = np.array(d["A_colmajor"]).reshape(nc, nr).T
    init = np.array(d["init"])[:50]
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A[:100, :50].copy()), 5, oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["strided_D"], orc["D"], rtol=1e-10)
    assert d["strided_iterations"] == orc["iterations"]


def test_dropin_user_matrices(dropin_output, oracle_mod):
    """A caller's own irlba::Matrix subclass (host products through its
    workspaces), a CenteredMatrix over it, and a gpu::DeviceMatrix whose
    products are device code, each against the oracle."""
    d = dropin_output
    nr, nc = 120, 70
    A = np.array(d["A_colmajor"]).reshape(nc, nr).T
    init = np.array(d["init"])
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 6, oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["user_D"], orc["D"], rtol=1e-10)
    assert d["user_iterations"] == orc["iterations"]
    cen = oracle_mod.compute(oracle_mod.Spec.dense(A, center=np.array(d["center"])), 4,
                             oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["user_centered_D"], cen["D"], rtol=1e-10)
    assert d["user_centered_iterations"] == cen["iterations"]
    assert "residual model is not fitted" in d["user_error_message"]
    x, i, p = np.array(d["sparse_x"]), np.array(d["sparse_i"], dtype=np.int32), np.array(d["sparse_p"], dtype=np.int64)
    sp = oracle_mod.compute(oracle_mod.Spec.sparse(nr, nc, x, i, p, True, 1), 4, oracle_mod.options(initial=init))
    np.testing.assert_allclose(d["device_D"], sp["D"], rtol=1e-10)
    assert d["device_iterations"] == sp["iterations"]
