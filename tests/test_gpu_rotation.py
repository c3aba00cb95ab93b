"""The restart step's basis rotation (compute.hpp:268-280: V <- V BV,
W <- W BU) on the tensor cores, through the C ABI, against an exact product.

FP64 form: every row of Q and column of R is scaled by a power of two and cut
into seven exact integer digit slices whose products are summed exactly, so the
error is bounded by 2^-50 (sum_j |Q[r, j]| |R[j, c]| + w max_j |Q[r, j]|
max_j |R[j, c]|), the level of an FP64 dot product of 64 terms. FP32 form:
three-term BF16 splits added into one FP32 accumulator (the rounding of an
FP32 dot product; each of the 6 slice pairs of each of the 4 K-steps adds once
to the accumulator): (2 w + 8) u sum_j |Q[r, j]| |R[j, c]|, u = 2^-24. The
CUDA-core kernels are held to the classical dot-product bound
(w + 3) u sum_j |Q[r, j]| |R[j, c]| (u = 2^-24 or 2^-53). The exact product is
a long-double matmul on up to 5,000 of the rows (the first and last 2,000 and
a random 1,000)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rotate(engine, fp64, Q, R, k, engine_id, ldq_pad=None, fcol=None, fnorm=None, inplace=False):
    """out[:, :k] = Q R[:, :k] (+ out[:, k] = fcol / fnorm) on the GPU; Q is
    L x w (numpy), column-major in device memory with leading dimension
    L + ldq_pad, or L rounded up to 32 (the engine's layout, 128-byte aligned
    columns) when ldq_pad is None."""
    import torch
    lib = engine.load_library()
    L, w = Q.shape
    dt = torch.float64 if fp64 else torch.float32
    ldq = (L + 31) // 32 * 32 if ldq_pad is None else L + ldq_pad
    cols = max(w, k + 1)
    Qp = np.zeros((cols, ldq))
    Qp[:w, :L] = Q.T
    Qd = torch.tensor(Qp, dtype=dt, device="cuda")
    Rd = torch.tensor(np.ascontiguousarray(R.T), dtype=torch.float64, device="cuda")   # column-major, ld w
    out = Qd if inplace else torch.full((cols, ldq), float("nan"), dtype=dt, device="cuda")
    fd = torch.tensor(fcol, dtype=dt, device="cuda") if fcol is not None else None
    nd = torch.tensor([fnorm], dtype=torch.float64, device="cuda") if fcol is not None else None
    st = lib.irlba_gb300_rotate_device(int(fp64), Qd.data_ptr(), L, ldq, w, Rd.data_ptr(), R.shape[0], k,
                                       out.data_ptr(), ldq, fd.data_ptr() if fd is not None else None,
                                       nd.data_ptr() if nd is not None else None, engine_id, None)
    assert st == 0, lib.irlba_gb300_last_error().decode()
    torch.cuda.synchronize()
    o = out.cpu().numpy().astype(np.float64)
    return o[:k + (1 if fcol is not None else 0), :L].T


def _rows(L):
    if L <= 5000:
        return np.arange(L)
    rng = np.random.default_rng(L)
    mid = rng.choice(np.arange(2000, L - 2000), size=1000, replace=False)
    return np.unique(np.concatenate([np.arange(2000), mid, np.arange(L - 2000, L)]))


def _bounds(Q, R, k, fp64, rows):
    q, r = Q[rows], R[:, :k]
    w = Q.shape[1]
    ref = (q.astype(np.longdouble) @ r.astype(np.longdouble)).astype(np.float64)
    sigma = np.abs(q) @ np.abs(r)
    mx = np.outer(np.abs(q).max(axis=1), np.abs(r).max(axis=0))
    if fp64:
        tc, u = 2.0 ** -50 * (sigma + w * mx), 2.0 ** -53
    else:
        u = 2.0 ** -24
        tc = (2 * w + 8) * u * sigma
    return ref, {1: tc, 0: (w + 3) * u * sigma}


def _check(engine, fp64, Q, R, k, **kw):
    rows = _rows(Q.shape[0])
    ref, bound = _bounds(Q, R, k, fp64, rows)
    for eng_id in (1, 0):
        got = _rotate(engine, fp64, Q, R, k, eng_id, **kw)[rows, :k]
        err = np.abs(got - ref)
        worst = np.max(err / np.maximum(bound[eng_id], 1e-300))
        assert np.all(err <= bound[eng_id]), "engine %d: worst error %.3f x bound" % (eng_id, worst)


def _orthogonal(w, seed):
    q, _ = np.linalg.qr(np.random.default_rng(seed).standard_normal((w, w)))
    return q


@pytest.mark.parametrize("fp64", [False, True])
@pytest.mark.parametrize("L,w,k,pad", [(300001, 57, 50, None), (300001, 57, 50, 3), (5, 3, 2, None), (5, 3, 2, 0),
                                       (4096, 64, 64, None), (1000, 17, 16, 1), (129, 33, 1, None)])
def test_rotation_matches_exact_product(engine, fp64, L, w, k, pad):
    # pad None: aligned columns (the FP32 kernel stages tiles with cp.async);
    # otherwise ldq = L + pad (direct loads).
    rng = np.random.default_rng(L + 7 * w)
    Q = rng.standard_normal((L, w)) / np.sqrt(L)
    if not fp64:
        Q = Q.astype(np.float32).astype(np.float64)
    R = _orthogonal(w, w)
    _check(engine, fp64, Q, R, k, ldq_pad=pad)


@pytest.mark.parametrize("fp64", [False, True])
def test_rotation_rows_of_mixed_magnitude(engine, fp64):
    # Rows spanning many binades, zero rows, single nonzero rows; columns of R
    # with one dominant entry.
    rng = np.random.default_rng(11)
    L, w, k = 2000, 40, 30
    Q = rng.standard_normal((L, w)) * np.exp2(rng.integers(-30, 30, size=(L, w)))
    Q[5] = 0.0
    Q[6] = 0.0
    Q[6, 3] = -1.5e-7
    Q[7, :] = 1e-300 if fp64 else 1e-30
    if not fp64:
        Q = Q.astype(np.float32).astype(np.float64)
    R = _orthogonal(w, 3)
    R[:, 2] *= np.exp2(rng.integers(-8, 8, size=w))
    _check(engine, fp64, Q, R, k)


def test_fp64_rotation_digit_bound(engine):
    # Every digit of every value at its maximum (mantissas of all ones) with
    # w = 64: the largest exact accumulator sums the kernel relies on.
    L, w, k = 256, 64, 64
    x = 1.0 - 2.0 ** -53
    Q = np.full((L, w), x)
    Q[1::2] *= -1.0
    R = np.full((w, w), x)
    R[:, 1::2] *= -1.0
    _check(engine, True, Q, R, k)


@pytest.mark.parametrize("fp64", [False, True])
def test_rotation_in_place_with_residual_column(engine, fp64):
    # The engine's call: V[:, :k] = V BV[:, :k] in place, V[:, k] = F / ||F||.
    rng = np.random.default_rng(5)
    L, w, k = 70001, 57, 48
    Q = rng.standard_normal((L, w)) / np.sqrt(L)
    F = rng.standard_normal(L)
    if not fp64:
        Q = Q.astype(np.float32).astype(np.float64)
        F = F.astype(np.float32).astype(np.float64)
    R = _orthogonal(w, 9)
    nrm = float(np.linalg.norm(F))
    rows = _rows(L)
    ref, bound = _bounds(Q, R, k, fp64, rows)
    for eng_id in (1, 0):
        got = _rotate(engine, fp64, Q, R, k, eng_id, fcol=F, fnorm=nrm, inplace=True)
        assert np.all(np.abs(got[rows, :k] - ref) <= bound[eng_id])
        np.testing.assert_allclose(got[:, k], F / nrm, rtol=1e-6 if not fp64 else 1e-15)


def test_rotation_engine_rejects_wide_bases(engine):
    import torch
    lib = engine.load_library()
    Q = torch.zeros(100 * 70, dtype=torch.float64, device="cuda")
    R = torch.zeros(70 * 70, dtype=torch.float64, device="cuda")
    st = lib.irlba_gb300_rotate_device(1, Q.data_ptr(), 100, 100, 70, R.data_ptr(), 70, 60, Q.data_ptr(), 100,
                                       None, None, 1, None)
    assert st == engine.ERROR_UNSUPPORTED


@pytest.mark.parametrize("fp64", [False, True])
def test_compute_same_with_either_rotation_engine(engine, oracle_mod, fp64):
    # A whole solve with tensor-core and with CUDA-core rotations: the FP64 form
    # matches the oracle (1e-10, identical restart counts) either way.
    from conftest import column_sines
    rng = np.random.default_rng(21)
    A = rng.standard_normal((3000, 400))
    init = rng.standard_normal(400)
    form = engine.FORM_FP64 if fp64 else engine.FORM_FP32_FP64STEPS
    res = []
    try:
        for eng_id in (1, 0):
            engine.set_rotation_engine(eng_id)
            res.append(engine.compute_simple(A, 20, engine.Options(initial=init), form=form))
    finally:
        engine.set_rotation_engine(1)
    orc = oracle_mod.compute(oracle_mod.Spec.dense(A), 20, oracle_mod.options(initial=init))
    for r in res:
        if fp64:
            np.testing.assert_allclose(r.D, orc["D"], rtol=1e-10, atol=0)
            assert r.iterations == orc["iterations"]
            assert np.max(column_sines(r.V, orc["V"])) < 1e-8
        else:
            np.testing.assert_allclose(r.D, orc["D"], rtol=1e-6, atol=0)
