"""Oracle for the differentiation form (test infrastructure only).

The reference has no derivative of irlba::compute / pca, so this restates the
mathematics the GPU adjoint implements, in dense numpy FP64, from a full
LAPACK SVD; it is pinned against central finite differences by
tests/test_adjoint_oracle.py.

truncated_svd_grad: dL/dA for (U, S, V) = top-k SVD of A, given the cotangents
gU, gS, gV (Townsend 2016 for the in-subspace F-matrix terms; the
orthogonal-complement terms from the first-order perturbation of singular
vectors, solved exactly against A_perp = (I - UU^T) A (I - VV^T), or with
exact=False the rank-k projection terms (I - UU^T) gU S^-1 V^T +
U S^-1 gV^T (I - VV^T)).

pca_operator / sparse_pca_grad: pca()'s centred and scaled operator
(pca.hpp:85-126: column means, standard deviations with m - 1, zero variance
-> 1) and the chain rule from dL/dA' back to the stored values of a sparse A,
with or without the statistics' dependence on the values.
"""
import numpy as np


def top_k_svd(A, k):
    U, s, Vt = np.linalg.svd(A, full_matrices=False)
    return U[:, :k], s[:k], Vt[:k].T


def truncated_svd_grad(A, k, gU=None, gS=None, gV=None, exact=True):
    m, n = A.shape
    U, S, V = top_k_svd(A, k)
    gU = np.zeros((m, k)) if gU is None else gU
    gS = np.zeros(k) if gS is None else gS
    gV = np.zeros((n, k)) if gV is None else gV
    T1 = U.T @ gU
    T2 = V.T @ gV
    s2 = S ** 2
    den = s2[None, :] - s2[:, None]
    F = np.zeros((k, k))
    off = ~np.eye(k, dtype=bool)
    F[off] = 1.0 / den[off]
    M = np.diag(gS) + (F * (T1 - T1.T)) * S[None, :] + S[:, None] * (F * (T2 - T2.T))
    Pu = np.eye(m) - U @ U.T
    Pv = np.eye(n) - V @ V.T
    bu = Pu @ gU
    bv = Pv @ gV
    Ap = Pu @ A @ Pv
    Y = np.zeros((m, k))
    Z = np.zeros((n, k))
    for j in range(k):
        if exact:
            Y[:, j] = np.linalg.solve(s2[j] * np.eye(m) - Ap @ Ap.T, bu[:, j])
            Z[:, j] = np.linalg.solve(s2[j] * np.eye(n) - Ap.T @ Ap, bv[:, j])
        else:
            Y[:, j] = bu[:, j] / s2[j]
            Z[:, j] = bv[:, j] / s2[j]
    X1 = U @ M + Y * S[None, :] + Ap @ Z
    X2 = Z * S[None, :] + Ap.T @ Y
    return X1 @ V.T + U @ X2.T


def pca_operator(A, center, scale):
    """(A', c, s) of pca.hpp:85-126 for a dense A (zeros included)."""
    m, n = A.shape
    c = A.mean(axis=0) if center else np.zeros(n)
    s = np.ones(n)
    if scale:
        var = ((A - c) ** 2).sum(axis=0)
        s = np.where(var != 0, np.sqrt(var / (m - 1)), 1.0)
    return (A - c) / s, c, s


def sparse_pca_grad(A, mask, center, scale, gAp, statistics=True):
    """dL/dA on the stored entries (mask) given dL/dA' = gAp for pca()'s
    operator A' = (A - 1 c^T) diag(1/s)."""
    m = A.shape[0]
    Ap, c, s = pca_operator(A, center, scale)
    g = gAp / s[None, :]
    if statistics and center:
        g = g - gAp.sum(axis=0)[None, :] / (m * s[None, :])
    if statistics and scale:
        q = (gAp * Ap).sum(axis=0)
        g = g - Ap * (q / ((m - 1) * s))[None, :]
    return np.where(mask, g, 0.0)
