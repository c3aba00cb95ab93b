"""CPU pins of the differentiation form's oracle (oracle/svd_adjoint.py):
central finite differences and torch's FP64 autograd through a full SVD."""
import numpy as np
import pytest

from oracle import svd_adjoint as sa


def _loss_parts(m, n, k, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((m, k)), rng.standard_normal((n, k)), rng.uniform(0.5, 1.5, k)


def _loss(A, k, G, H, w):
    U, S, V = sa.top_k_svd(A, k)
    return float(w @ S + np.sum((G.T @ U) ** 2) + np.sum((H.T @ V) ** 2))


def _cotangents(A, k, G, H, w):
    U, S, V = sa.top_k_svd(A, k)
    return 2 * G @ (G.T @ U), w.copy(), 2 * H @ (H.T @ V)


def _fd(f, A, E, h=1e-6):
    return (f(A + h * E) - f(A - h * E)) / (2 * h)


@pytest.mark.parametrize("m,n,k", [(14, 9, 3), (9, 14, 4), (30, 12, 5)])
def test_truncated_grad_matches_finite_differences(m, n, k):
    rng = np.random.default_rng(m * n + k)
    A = rng.standard_normal((m, n))
    G, H, w = _loss_parts(m, n, k, 1)
    gU, gS, gV = _cotangents(A, k, G, H, w)
    grad = sa.truncated_svd_grad(A, k, gU, gS, gV)
    for t in range(4):
        E = rng.standard_normal((m, n))
        fd = _fd(lambda X: _loss(X, k, G, H, w), A, E)
        assert abs(np.sum(grad * E) - fd) <= 1e-6 * max(1.0, abs(fd))


def test_projection_terms_need_rank_k():
    """The rank-k projection terms are exact for a rank-k matrix and off for a
    full-rank one; the complement solve is exact for both."""
    rng = np.random.default_rng(3)
    m, n, k = 20, 10, 3
    G, H, w = _loss_parts(m, n, k, 2)
    low = rng.standard_normal((m, k)) @ rng.standard_normal((k, n))
    full = low + 0.3 * rng.standard_normal((m, n))
    for A, close in ((low, True), (full, False)):
        gU, gS, gV = _cotangents(A, k, G, H, w)
        exact = sa.truncated_svd_grad(A, k, gU, gS, gV, exact=True)
        proj = sa.truncated_svd_grad(A, k, gU, gS, gV, exact=False)
        rel = np.linalg.norm(exact - proj) / np.linalg.norm(exact)
        assert (rel < 1e-8) == close


def test_truncated_grad_matches_torch_full_svd():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(7)
    m, n, k = 40, 16, 5
    A = rng.standard_normal((m, n))
    G, H, w = _loss_parts(m, n, k, 4)
    At = torch.tensor(A, requires_grad=True)
    U, S, Vh = torch.linalg.svd(At, full_matrices=False)
    L = (torch.tensor(w) * S[:k]).sum() + ((torch.tensor(G).T @ U[:, :k]) ** 2).sum() + \
        ((torch.tensor(H).T @ Vh[:k].T) ** 2).sum()
    L.backward()
    gU, gS, gV = _cotangents(A, k, G, H, w)
    ours = sa.truncated_svd_grad(A, k, gU, gS, gV)
    np.testing.assert_allclose(ours, At.grad.numpy(), rtol=1e-9, atol=1e-9 * np.abs(ours).max())


@pytest.mark.parametrize("center,scale", [(True, True), (True, False), (False, True)])
def test_sparse_pca_grad_matches_finite_differences(center, scale):
    rng = np.random.default_rng(11)
    m, n, k = 25, 7, 2
    mask = rng.random((m, n)) < 0.4
    A = np.where(mask, rng.standard_normal((m, n)) + 1.0, 0.0)
    G, H, w = _loss_parts(m, n, k, 5)

    def loss_of(X):
        Ap, _, _ = sa.pca_operator(X, center, scale)
        return _loss(Ap, k, G, H, w)

    Ap, _, _ = sa.pca_operator(A, center, scale)
    gU, gS, gV = _cotangents(Ap, k, G, H, w)
    gAp = sa.truncated_svd_grad(Ap, k, gU, gS, gV)
    grad = sa.sparse_pca_grad(A, mask, center, scale, gAp, statistics=True)
    for t in range(4):
        E = np.where(mask, rng.standard_normal((m, n)), 0.0)
        fd = _fd(loss_of, A, E)
        assert abs(np.sum(grad * E) - fd) <= 1e-6 * max(1.0, abs(fd))
