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


@pytest.mark.parametrize("L,ncols", [(10000, 25), (300000, 57)])
def test_noalloc_matches_allocating_entry_point(engine, L, ncols):
    import torch
    lib = _lib(engine)
    rng = np.random.default_rng(L + ncols)
    Q, _ = np.linalg.qr(rng.standard_normal((L, ncols + 3)))
    Qd = torch.tensor(np.asfortranarray(Q).T.copy(), device="cuda")  # column j contiguous, ld = L
    v0 = rng.standard_normal(L)

    ref = torch.tensor(v0, device="cuda")
    assert lib.irlba_gb300_orthogonalize_vector_device(Qd.data_ptr(), L, L, ncols, ref.data_ptr(), None) == 0
    torch.cuda.synchronize()
    ref = ref.cpu().numpy()

    for call in range(2):
        v = torch.tensor(v0, device="cuda")
        st = lib.irlba_gb300_orthogonalize_vector_device_noalloc(Qd.data_ptr(), L, L, ncols, v.data_ptr(), None)
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
