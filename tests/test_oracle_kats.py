"""The oracle pinned to CppIrlba's own known-answer tests and to LAPACK.

KATs come from tests/golden/reference_kats.json (extracted from the reference's
tests/src/lanczos.cpp and tests/src/compute.cpp by tests/golden/make_golden.py).
Eigen's JacobiSVD is replaced by LAPACK (numpy) as the exact-SVD yardstick, with
the tolerances of the reference's tests.
"""
import json
import os

import numpy as np
import pytest

from conftest import column_sines, normal_matrix, same_same, simulate_compressed_sparse

KATS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_kats.json")))


def test_cgs_kat(oracle_mod):
    # tests/src/lanczos.cpp:11-52
    m = np.array(KATS["cgs_basis_rowmajor_5x4"]).reshape(5, 4)
    v = np.array(KATS["cgs_vector"])
    out = oracle_mod.orthogonalize_vector(m, v, 4)
    assert np.sum(out ** 2) > 0.1
    for i in range(4):
        # The reference's loop (lanczos.cpp:40-46) never advances its column
        # iterator, so what it asserts is sum(out) * m(0, i) < 1e-10.
        assert np.sum(out) * m[0, i] < 1e-10
        # The basis is printed to 7 digits, so it is orthonormal to ~1e-7 only.
        assert abs(out @ m[:, i]) < 1e-6
    out2 = oracle_mod.orthogonalize_vector(m, v, 2)
    assert not np.array_equal(out, out2)


def test_requested_ge_half_smaller_kat(oracle_mod):
    # tests/src/compute.cpp:33-41
    for req, smaller, expected in KATS["requested_ge_half_smaller"]:
        assert oracle_mod.requested_ge_half_smaller(req, smaller) == expected


def test_choose_work_kat(oracle_mod):
    # tests/src/compute.cpp:43-50
    for req, extra, smaller, expected in KATS["choose_requested_plus_extra_work_or_smaller"]:
        assert oracle_mod.choose_work(req, extra, smaller) == expected


def test_update_k_kat(oracle_mod):
    # tests/src/compute.cpp:52-76, 5^4 grid against R irlba's convtests() logic
    for k, req, conv, work, expected in KATS["update_k"]:
        assert oracle_mod.update_k(k, req, conv, work) == expected


@pytest.mark.parametrize("shape", [(20, 10), (10, 20), (57, 57), (100, 7), (3, 40), (1, 1)])
def test_svd_matches_lapack(oracle_mod, shape):
    A = normal_matrix(*shape, seed=sum(shape))
    U, S, V = oracle_mod.svd(A)
    ref = np.linalg.svd(A, compute_uv=False)
    np.testing.assert_allclose(S, ref, rtol=1e-13, atol=1e-13 * ref[0])
    np.testing.assert_allclose(U @ np.diag(S) @ V.T, A, atol=1e-12 * ref[0])
    np.testing.assert_allclose(U.T @ U, np.eye(U.shape[1]), atol=1e-13)
    np.testing.assert_allclose(V.T @ V, np.eye(V.shape[1]), atol=1e-13)


def test_svd_rank_deficient_completion(oracle_mod):
    A = normal_matrix(12, 3) @ normal_matrix(3, 9, seed=7)
    U, S, V = oracle_mod.svd(A)
    assert np.all(S[3:] < 1e-12 * S[0])
    np.testing.assert_allclose(U.T @ U, np.eye(9), atol=1e-12)
    np.testing.assert_allclose(U @ np.diag(S) @ V.T, A, atol=1e-12 * S[0])


def _restart_shaped(n, k, seed):
    # The shape of B after a restart (compute.hpp:282-293 then the Lanczos run):
    # diagonal singular values, a residual column k, an upper-bidiagonal tail.
    rng = np.random.default_rng(seed)
    B = np.zeros((n, n))
    B[np.arange(k), np.arange(k)] = np.sort(rng.uniform(1, 100, k))[::-1]
    B[:k, k] = 1e-3 * rng.standard_normal(k)
    for i in range(k, n):
        B[i, i] = abs(rng.standard_normal())
        if i + 1 < n:
            B[i, i + 1] = abs(rng.standard_normal())
    return B


@pytest.mark.parametrize("case", ["1", "2", "7", "57", "64", "restart", "rank2", "zero", "ties"])
def test_svd_square_two_sided(oracle_mod, case):
    # The restart SVD (two-sided Jacobi as Eigen::JacobiSVD, compute.hpp:225).
    if case == "restart":
        A = _restart_shaped(57, 50, 3)
    elif case == "rank2":
        A = normal_matrix(30, 2, seed=4) @ normal_matrix(2, 30, seed=5)
    elif case == "zero":
        A = np.zeros((5, 5))
    elif case == "ties":
        A = np.diag([3.0, 1.0, 3.0, 2.0, 1.0])
    else:
        n = int(case)
        A = normal_matrix(n, n, seed=n)
    U, S, V = oracle_mod.svd_square(A)
    n = A.shape[0]
    ref = np.linalg.svd(A, compute_uv=False)
    top = max(ref[0], 1.0)
    np.testing.assert_allclose(S, ref, rtol=1e-13, atol=1e-13 * top)
    assert np.all(np.diff(S) <= 0)
    np.testing.assert_allclose(U @ np.diag(S) @ V.T, A, atol=1e-13 * top * max(n, 1))
    np.testing.assert_allclose(U.T @ U, np.eye(n), atol=1e-13)
    np.testing.assert_allclose(V.T @ V, np.eye(n), atol=1e-13)
    # canonical signs: the largest-magnitude entry of each V column is positive
    for j in range(n):
        assert V[np.argmax(np.abs(V[:, j])), j] > 0


def _lanczos_setup(nr, nc, work):
    rng = np.random.default_rng(42)
    A = rng.standard_normal((nr, nc))
    V = np.zeros((nc, work))
    V[:, 0] = rng.standard_normal(nc)
    V[:, 0] /= np.linalg.norm(V[:, 0])
    return A, np.zeros((nr, work)), V, np.zeros((work, work))


@pytest.mark.parametrize("nr", [10, 20, 30])
@pytest.mark.parametrize("nc", [10, 20, 30])
@pytest.mark.parametrize("work", [3, 5, 7])
def test_lanczos_orthogonality(oracle_mod, nr, nc, work):
    # tests/src/lanczos.cpp:85-117
    A, W, V, B = _lanczos_setup(nr, nc, work)
    W, V, B, F = oracle_mod.lanczos(oracle_mod.Spec.dense(A), W, V, B, 0)
    for Q in (W, V):
        G = Q.T @ Q
        assert np.allclose(np.diag(G), 1.0, atol=1e-12)
        off = G - np.diag(np.diag(G))
        assert np.max(np.abs(off)) < 1e-11


@pytest.mark.parametrize("nr,nc,work", [(10, 10, 7), (30, 20, 5), (20, 30, 7)])
def test_lanczos_restart_equivalence(oracle_mod, nr, nc, work):
    # tests/src/lanczos.cpp:119-163: restarting at mid equals one full run.
    A, W, V, B = _lanczos_setup(nr, nc, work)
    spec = oracle_mod.Spec.dense(A)
    mid = work // 2
    sW, sV, sB, F = oracle_mod.lanczos(spec, W[:, :mid], V[:, :mid], B[:mid, :mid], 0)
    cW = np.zeros((nr, work)); cW[:, :mid] = sW
    cV = np.zeros((nc, work)); cV[:, :mid] = sV
    cB = np.zeros((work, work)); cB[:mid, :mid] = sB
    cV[:, mid] = F / np.linalg.norm(F)
    cW, cV, cB, _ = oracle_mod.lanczos(spec, cW, cV, cB, mid)
    fW, fV, fB, _ = oracle_mod.lanczos(spec, W, V, B, 0)
    np.testing.assert_allclose(cW, fW, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(cV, fV, rtol=1e-6, atol=1e-9)


def test_compute_vs_exact(oracle_mod):
    # tests/src/compute.cpp:15-31 (rank + workspace > min dim -> near exact)
    A = normal_matrix(20, 10)
    r = oracle_mod.compute(oracle_mod.Spec.dense(A), 5, oracle_mod.options(exact_for_large_number=0))
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    np.testing.assert_allclose(r["D"], S[:5], rtol=1e-8)
    assert np.max(column_sines(r["U"], U[:, :5])) < 1e-8
    assert np.max(column_sines(r["V"], Vt[:5].T)) < 1e-8


@pytest.mark.parametrize("nr", [20, 50, 100])
@pytest.mark.parametrize("nc", [20, 50, 100])
@pytest.mark.parametrize("rank", [2, 5, 10])
def test_compute_sweep(oracle_mod, nr, nc, rank):
    # tests/src/compute.cpp:78-123: tol 1e-9 -> 1e-6 agreement with the exact SVD
    A = normal_matrix(nr, nc)
    r = oracle_mod.compute(oracle_mod.Spec.dense(A), rank, oracle_mod.options(convergence_tolerance=1e-9))
    U, S, Vt = np.linalg.svd(A, full_matrices=False)
    np.testing.assert_allclose(r["D"], S[:rank], rtol=1e-6)
    assert np.max(column_sines(r["U"], U[:, :rank])) < 1e-5
    assert np.max(column_sines(r["V"], Vt[:rank].T)) < 1e-5
    init = np.random.default_rng(1239 + nr + nc + rank).standard_normal(nc)
    r2 = oracle_mod.compute(oracle_mod.Spec.dense(A), rank,
                            oracle_mod.options(convergence_tolerance=1e-9, initial=init))
    np.testing.assert_allclose(r["D"], r2["D"], rtol=1e-6)


def test_exact_fallbacks(oracle_mod):
    # tests/src/compute.cpp:157-191
    small = normal_matrix(10, 3)
    r = oracle_mod.compute(oracle_mod.Spec.dense(small), 2)
    assert r["iterations"] == 0 and r["converged"]
    np.testing.assert_allclose(r["D"], np.linalg.svd(small, compute_uv=False)[:2], rtol=1e-13)
    mat = normal_matrix(20, 50)
    S = np.linalg.svd(mat, compute_uv=False)
    r = oracle_mod.compute(oracle_mod.Spec.dense(mat), 15)
    np.testing.assert_allclose(r["D"], S[:15], rtol=1e-13)
    r = oracle_mod.compute(oracle_mod.Spec.dense(mat), 20)
    np.testing.assert_allclose(r["D"], S, rtol=1e-12)
    r = oracle_mod.compute(oracle_mod.Spec.dense(mat), 50, oracle_mod.options(cap_number=1))
    assert r["D"].shape == (20,)


def test_compute_errors(oracle_mod):
    # tests/src/compute.cpp:193-238
    spec = oracle_mod.Spec.dense(normal_matrix(20, 10))
    with pytest.raises(oracle_mod.OracleError, match="cannot be greater than"):
        oracle_mod.compute(spec, 100)
    with pytest.raises(oracle_mod.OracleError, match="must be less than"):
        oracle_mod.compute(spec, 10, oracle_mod.options(exact_for_large_number=0))
    with pytest.raises(oracle_mod.OracleError, match="must be positive"):
        oracle_mod.compute(spec, 0, oracle_mod.options(extra_work=0))
    with pytest.raises(oracle_mod.OracleError, match="^initialization"):
        oracle_mod.compute(spec, 2, oracle_mod.options(initial=np.zeros(1)))


@pytest.mark.parametrize("nr", [10, 49, 97])
@pytest.mark.parametrize("nc", [10, 51, 88])
@pytest.mark.parametrize("nt", [1, 3])
def test_parallel_sparse(oracle_mod, nr, nc, nt):
    # tests/src/Matrix/sparse.cpp:44-149
    dense, x, i, p = simulate_compressed_sparse(nr, nc)
    csc = oracle_mod.Spec.sparse(nr, nc, x, i, p, True, nt)
    xr, ir, pr = _csr(dense)
    csr = oracle_mod.Spec.sparse(nc, nr, x, i, p, False, nt)  # the transpose, stored CSR
    np.testing.assert_array_equal(oracle_mod.realize(csc), dense)
    np.testing.assert_array_equal(oracle_mod.realize(csr).T, dense)
    vec = np.random.default_rng(nr * nc * nt // 10).standard_normal(nc)
    ref = dense @ vec
    np.testing.assert_allclose(oracle_mod.multiply(csc, vec), ref, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle_mod.adjoint_multiply(csr, vec), ref, rtol=1e-12, atol=1e-12)
    vec2 = np.random.default_rng(nr * nc * nt // 20).standard_normal(nr)
    ref2 = dense.T @ vec2
    np.testing.assert_allclose(oracle_mod.adjoint_multiply(csc, vec2), ref2, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(oracle_mod.multiply(csr, vec2), ref2, rtol=1e-12, atol=1e-12)
    if nt > 1:
        pb, sb, snz = oracle_mod.partitions(csc, nt)
        assert pb[0] == 0 and sb[0] == 0 and pb[-1] == nc and sb[-1] == nr
        assert np.all(np.diff(pb) >= 0) and np.all(np.diff(sb) >= 0)
        np.testing.assert_array_equal(snz[0], p[:-1])
        np.testing.assert_array_equal(snz[-1], p[1:])
        for t in range(nt):
            for c in range(nc):
                first, last = snz[t, c], snz[t + 1, c]
                assert first <= last
                if first != last:
                    assert i[first] >= sb[t] and i[last - 1] < sb[t + 1]


def _csr(dense):
    from conftest import to_csr
    return to_csr(dense)


def test_random_normals(oracle_mod):
    # tests/src/utils.cpp:21-65
    a = oracle_mod.random_normals(10, 1000)
    assert np.all(a != 0) and len(np.unique(a)) == 10
    b = oracle_mod.random_normals(11, 1000)
    assert np.all(b != 0) and len(np.unique(b)) == 11
    np.testing.assert_array_equal(a, oracle_mod.random_normals(10, 1000))


def _spawn(A):
    mean = A.mean(axis=0)
    centered = A - mean
    both = centered / np.sqrt((centered ** 2).sum(axis=0) / (A.shape[0] - 1))
    scaled = A / np.sqrt((A ** 2).sum(axis=0) / (A.shape[0] - 1))
    return centered, scaled, both


@pytest.mark.parametrize("nr,nc,rank", [(20, 20, 2), (50, 100, 5), (100, 50, 10), (100, 100, 5)])
def test_pca_identities(oracle_mod, nr, nc, rank):
    # tests/src/pca.cpp:66-141
    A = normal_matrix(nr, nc)
    centered, scaled, both = _spawn(A)
    for center, scale, ref in ((True, True, both), (True, False, centered), (False, True, scaled), (False, False, A)):
        res = oracle_mod.pca(oracle_mod.Spec.dense(A), center, scale, rank)
        res2 = oracle_mod.compute(oracle_mod.Spec.dense(ref), rank)
        np.testing.assert_allclose(res["variances"], res2["D"] ** 2 / (nr - 1), rtol=1e-8)
        assert np.max(column_sines(res["rotation"], res2["V"])) < 1e-7
        if center:
            for i in range(rank):
                assert abs(res["scores"][:, i].sum()) < 1e-8
                assert same_same(np.sum(res["scores"][:, i] ** 2) / (nr - 1), res["variances"][i], 1e-8)


def test_pca_sparse_equals_dense(oracle_mod):
    # tests/src/pca.cpp:218-240
    dense, x, i, p = simulate_compressed_sparse(76, 128)
    rd = oracle_mod.pca(oracle_mod.Spec.dense(dense), True, True, 8)
    rs = oracle_mod.pca(oracle_mod.Spec.sparse(76, 128, x, i, p, True, 1), True, True, 8)
    np.testing.assert_allclose(rd["variances"], rs["variances"], rtol=1e-8)
    assert np.max(column_sines(rd["rotation"], rs["rotation"])) < 1e-7
    for j in range(8):
        assert abs(rs["scores"][:, j].sum()) < 1e-8


def test_pca_errors(oracle_mod):
    with pytest.raises(oracle_mod.OracleError, match="cannot center"):
        oracle_mod.pca(oracle_mod.Spec.dense(np.zeros((0, 10))), True, True, 1)
    with pytest.raises(oracle_mod.OracleError, match="cannot scale"):
        oracle_mod.pca(oracle_mod.Spec.dense(normal_matrix(1, 10)), True, True, 1)
    out = oracle_mod.pca(oracle_mod.Spec.dense(np.zeros((10, 2))), True, True, 1)
    assert out["converged"] and np.all(np.isfinite(out["scores"])) and np.all(np.isfinite(out["rotation"]))


@pytest.mark.parametrize("rank", [2, 5, 10])
def test_invariant_subspace(oracle_mod, rank):
    # tests/src/invariant.cpp:7-86
    rng = np.random.default_rng(42)
    A = np.zeros((100, 50))
    A[:, :rank] = rng.standard_normal((100, rank))
    for i in range(rank, 50):
        A[:, i] = A[:, i % rank]
    r = oracle_mod.compute(oracle_mod.Spec.dense(A), rank + 3)
    assert np.all(r["D"][:rank] > 0.01)
    assert np.all(r["D"][rank:] < 1e-8)
    r = oracle_mod.compute(oracle_mod.Spec.dense(A), rank + 2)
    rec = r["U"] @ np.diag(r["D"]) @ r["V"].T
    np.testing.assert_allclose(rec, A, atol=1e-8 * np.abs(A).max())
