"""The allocation-free orthogonalize_vector entry point, for callers that cannot
call cudaMalloc/cudaFree (code inside another framework's memory budget, or
latency-critical loops where an allocation would synchronize the device).

Checked through the C ABI against the allocating entry point, on two calls in a
row (the shared scratch keeps the previous call's contents, so the second call
shows it is cleared correctly), plus the size limit. This file is collected
last so a run that stops at its first failure has run everything else."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, as the other FP64 GPU parity tests


def _lib(engine):
    lib = engine.load_library()
    fn = lib.irlba_gb300_orthogonalize_vector_device_noalloc
    fn.restype = ctypes.c_int32
    fn.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                   ctypes.c_void_p]
    return lib


@pytest.mark.parametrize("L,ncols,pad", [(10000, 25, 0), (300000, 57, 0), (20000, 40, 7)])
def test_noalloc_matches_allocating_entry_point(engine, L, ncols, pad):
    import torch
    lib = _lib(engine)
    rng = np.random.default_rng(L + ncols)
    Q, _ = np.linalg.qr(rng.standard_normal((L, ncols + 3)))
    ldq = L + pad
    Qp = np.zeros((ncols + 3, ldq))
    Qp[:, :L] = Q.T
    Qd = torch.tensor(Qp, device="cuda")  # column j contiguous, leading dimension ldq
    v0 = rng.standard_normal(L)

    ref = torch.tensor(v0, device="cuda")
    assert lib.irlba_gb300_orthogonalize_vector_device(Qd.data_ptr(), L, ldq, ncols, ref.data_ptr(), None) == 0
    torch.cuda.synchronize()
    ref = ref.cpu().numpy()

    for call in range(2):
        v = torch.tensor(v0, device="cuda")
        st = lib.irlba_gb300_orthogonalize_vector_device_noalloc(Qd.data_ptr(), L, ldq, ncols, v.data_ptr(), None)
        assert st == 0, lib.irlba_gb300_last_error().decode()
        torch.cuda.synchronize()
        out = v.cpu().numpy()
        np.testing.assert_allclose(out, ref, rtol=TOL, atol=TOL * np.abs(ref).max())
        # and the result is orthogonal to the basis it was projected against
        assert np.max(np.abs(Q[:, :ncols].T @ out)) < 1e-10


def test_noalloc_rejects_oversized_requests(engine):
    import torch
    lib = _lib(engine)
    L, ncols = 40_000_000, 1024  # needs far more than the fixed 1 MiB of scratch
    v = torch.zeros(4, dtype=torch.float64, device="cuda")
    st = lib.irlba_gb300_orthogonalize_vector_device_noalloc(v.data_ptr(), L, L, ncols, v.data_ptr(), None)
    assert st == engine.ERROR_INVALID_ARGUMENT
    assert "scratch" in lib.irlba_gb300_last_error().decode()


def test_noalloc_scratch_boundary(engine):
    """ncols = 256: the largest accepted L uses 128 + 256 + 510 * 256 = 130944
    of the 131072 scratch doubles; one more 256-row unit needs 131200 and is
    rejected. The buffers are sized for the rejected request as well, so every
    access stays inside them whichever way the check goes."""
    import torch
    lib = _lib(engine)
    ncols = 256
    L_ok = 256 * ((131072 - 128 - 256) // 256)
    L_bad = L_ok + 256
    rng = np.random.default_rng(5)
    Qd = torch.tensor(rng.standard_normal((ncols, L_bad)), device="cuda")  # ld = L_bad
    v0 = rng.standard_normal(L_bad)

    ref = torch.tensor(v0[:L_ok], device="cuda")
    assert lib.irlba_gb300_orthogonalize_vector_device(Qd.data_ptr(), L_ok, L_bad, ncols, ref.data_ptr(), None) == 0
    v = torch.tensor(v0[:L_ok], device="cuda")
    st = lib.irlba_gb300_orthogonalize_vector_device_noalloc(Qd.data_ptr(), L_ok, L_bad, ncols, v.data_ptr(), None)
    assert st == 0, lib.irlba_gb300_last_error().decode()
    torch.cuda.synchronize()
    r = ref.cpu().numpy()
    np.testing.assert_allclose(v.cpu().numpy(), r, rtol=TOL, atol=TOL * np.abs(r).max())

    w = torch.tensor(v0, device="cuda")
    st = lib.irlba_gb300_orthogonalize_vector_device_noalloc(Qd.data_ptr(), L_bad, L_bad, ncols, w.data_ptr(), None)
    assert st == engine.ERROR_INVALID_ARGUMENT
    assert "scratch" in lib.irlba_gb300_last_error().decode()
