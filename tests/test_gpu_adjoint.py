"""Differentiation form on the GPU, through the libtorch autograd Functions.

Loss L = sum_i w_i sigma_i + ||G^T U||_F^2 with seeded G and w (the
differentiable truncated-SVD workload: planted spectrum sigma_i = 50 / i plus
N(0, 0.01) noise). Checked against the FP64 oracle (oracle/svd_adjoint.py,
itself pinned to finite differences and to torch's autograd through a full
SVD), against central finite differences of the GPU forward, and against
torch's FP64 autograd through a full SVD for the FP32 4096 x 1024 case.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _ag():
    from cppirlba_gb300 import autograd
    autograd.load_extension()
    return autograd


def _loss_inputs(m, k, seed=21):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((m, k)), rng.uniform(0.5, 1.5, k)


def _torch_loss(U, S, G, w):
    return (w * S).sum() + ((G.T @ U) ** 2).sum()


def _oracle_grad(A, k, G, w, exact=True):
    from oracle import svd_adjoint as sa
    U, S, V = sa.top_k_svd(A, k)
    return sa.truncated_svd_grad(A, k, 2 * G @ (G.T @ U), w, None, exact=exact)


@pytest.mark.parametrize("k", [32, 10])
def test_dense_fp64_gradient_matches_oracle_and_fd(engine, k):
    from cppirlba_gb300 import datagen
    ag = _ag()
    A = datagen.adjoint_dense(256, 64, seed=8, dtype=np.float64)
    G, w = _loss_inputs(256, k)
    At = torch.tensor(A, device="cuda", requires_grad=True)
    Gt, wt = torch.tensor(G, device="cuda"), torch.tensor(w, device="cuda")
    U, S, V = ag.truncated_svd(At, k, tol=1e-12)
    _torch_loss(U, S, Gt, wt).backward()
    grad = At.grad.cpu().numpy()
    ref = _oracle_grad(A, k, G, w)
    assert np.linalg.norm(grad - ref) / np.linalg.norm(ref) < 1e-8
    rng = np.random.default_rng(4)

    def f(X):
        with torch.no_grad():
            Ux, Sx, _ = ag.truncated_svd(torch.tensor(X, device="cuda"), k, tol=1e-13)
            return float(_torch_loss(Ux, Sx, Gt, wt))

    h = 1e-5
    for _ in range(3):
        E = rng.standard_normal(A.shape)
        fd = (f(A + h * E) - f(A - h * E)) / (2 * h)
        assert abs(np.sum(grad * E) - fd) <= 1e-6 * max(1.0, abs(fd))


def test_projection_only_mode_matches_rank_k_formula(engine):
    from cppirlba_gb300 import datagen
    ag = _ag()
    A = datagen.adjoint_dense(200, 60, seed=9, dtype=np.float64)
    k = 8
    G, w = _loss_inputs(200, k, seed=5)
    At = torch.tensor(A, device="cuda", requires_grad=True)
    U, S, V = ag.truncated_svd(At, k, tol=1e-12, cg_tol=-1.0)
    _torch_loss(U, S, torch.tensor(G, device="cuda"), torch.tensor(w, device="cuda")).backward()
    ref = _oracle_grad(A, k, G, w, exact=False)
    grad = At.grad.cpu().numpy()
    assert np.linalg.norm(grad - ref) / np.linalg.norm(ref) < 1e-8
    exact = _oracle_grad(A, k, G, w, exact=True)
    assert np.linalg.norm(grad - exact) / np.linalg.norm(exact) > 1e-4


def test_dense_fp32_4096x1024_matches_fp64_full_svd_gradient(engine):
    from cppirlba_gb300 import datagen
    ag = _ag()
    k = 32
    A = datagen.adjoint_dense(4096, 1024, seed=5)
    G, w = _loss_inputs(4096, k, seed=6)
    At = torch.tensor(A, device="cuda", requires_grad=True)
    Gt32, wt32 = torch.tensor(G, device="cuda", dtype=torch.float32), torch.tensor(w, device="cuda", dtype=torch.float32)
    U, S, V = ag.truncated_svd(At, k, tol=1e-6)
    _torch_loss(U, S, Gt32, wt32).backward()
    grad = At.grad.double()
    Ar = torch.tensor(A, device="cuda", dtype=torch.float64, requires_grad=True)
    Ur, Sr, Vhr = torch.linalg.svd(Ar, full_matrices=False)
    _torch_loss(Ur[:, :k], Sr[:k], torch.tensor(G, device="cuda"), torch.tensor(w, device="cuda")).backward()
    rel = float(torch.linalg.norm(grad - Ar.grad) / torch.linalg.norm(Ar.grad))
    assert rel < 1e-3, rel
    rel_s = float(torch.max(torch.abs(S.detach().double() - Sr[:k].detach()) / Sr[:k].detach()))
    assert rel_s < 1e-5, rel_s


@pytest.mark.parametrize("column_major", [True, False])
@pytest.mark.parametrize("center,scale,statistics", [(True, True, True), (True, False, True), (False, True, True),
                                                     (True, True, False)])
def test_sparse_pca_gradient_matches_oracle(engine, column_major, center, scale, statistics):
    from cppirlba_gb300 import datagen
    from oracle import svd_adjoint as sa
    ag = _ag()
    inp = datagen.scrna_pca_input(60, 400, 0.25, 13, np.float64, cell_major=not column_major)
    assert inp.column_major == column_major
    dense = inp.to_dense()
    mask = dense != 0
    k = 5
    G, w = _loss_inputs(inp.nrow, k, seed=9)
    vals = torch.tensor(inp.val, device="cuda", requires_grad=True)
    U, S, V, c, s = ag.sparse_pca_svd(vals, inp.ptr, inp.idx, inp.nrow, inp.ncol, inp.column_major, center, scale, k,
                                      tol=1e-12, statistics=statistics)
    _torch_loss(U, S, torch.tensor(G, device="cuda"), torch.tensor(w, device="cuda")).backward()
    Ap, c0, s0 = sa.pca_operator(dense, center, scale)
    if center:
        np.testing.assert_allclose(c.cpu().numpy(), c0, rtol=1e-12, atol=1e-15)
    if scale:
        np.testing.assert_allclose(s.cpu().numpy(), s0, rtol=1e-12)
    gAp = _oracle_grad(Ap, k, G, w)
    ref_dense = sa.sparse_pca_grad(dense, mask, center, scale, gAp, statistics=statistics)
    # Stored order of the input: primary-major over (ptr, idx).
    prim = np.repeat(np.arange(len(inp.ptr) - 1), np.diff(inp.ptr))
    rows, cols = (inp.idx, prim) if column_major else (prim, inp.idx)
    ref = ref_dense[rows, cols]
    grad = vals.grad.cpu().numpy()
    assert np.linalg.norm(grad - ref) / np.linalg.norm(ref) < 1e-7
