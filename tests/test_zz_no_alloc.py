"""The allocation-free eigensolver entry point, cir_eigh_noalloc.

Callers that own the GPU memory budget (for example a simulation engine calling the
eigensolver from inside its own time step) cannot let the library allocate: cudaMalloc
and cudaFree synchronise the device and can fail in the middle of a run.
cir_eigh_noalloc works on the caller's device buffers and keeps its scratch in a fixed
8 MiB device array.  This file is collected last so that a failure here comes after every
other test has run; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sym(rng, n, scale=1000.0):
    a = rng.standard_normal((n, n))
    return ((a + a.T) * (scale / np.sqrt(8 * n))).astype(np.float32)


def _noalloc(lib, A):
    """cir_eigh_noalloc through the C ABI on device copies of A; returns (w, V) on the host."""
    import torch
    from calcir_gb300._lib import check, load
    nmat, n = A.shape[0], A.shape[-1]
    dA = torch.from_numpy(np.ascontiguousarray(A)).cuda()
    dw = torch.empty((nmat, n), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    check(load().cir_eigh_noalloc(nmat, n, C.c_void_p(dA.data_ptr()), C.c_void_p(dw.data_ptr()), None))
    V = np.ascontiguousarray(np.swapaxes(dA.cpu().numpy(), 1, 2))   # column j = eigenvector j
    return dw.cpu().numpy(), V


@pytest.mark.parametrize("n,nmat", [(130, 3), (256, 2)])
def test_noalloc_matches_cir_eigh_twice(lib, n, nmat):
    """Two calls in a row agree with cir_eigh (the allocating entry point) within the
    eigensolver tolerance used by the other tests."""
    rng = np.random.default_rng(n)
    for call in range(2):
        A = np.stack([_sym(rng, n) for _ in range(nmat)])
        w0, V0 = _noalloc(lib, A)
        with lib.Engine(lib.default_params(species="H2O"), 8) as eng:
            w1, V1 = eng.eigh(A)
        for m in range(nmat):
            nrm = np.abs(w1[m]).max()
            assert np.abs(w0[m] - w1[m]).max() <= 2e-6 * nrm * max(1.0, np.sqrt(n) / 4), (call, m)
            # the same subspaces: V0 diag(w) V0^T reproduces A like V1 does
            R0 = (V0[m].astype(np.float64) * w0[m]) @ V0[m].T.astype(np.float64)
            assert np.abs(R0 - A[m]).max() <= 4e-6 * nrm * max(1.0, np.sqrt(n) / 4), (call, m)
            assert np.abs(V0[m].T.astype(np.float64) @ V0[m] - np.eye(n)).max() <= 2e-6 * max(1.0, np.sqrt(n))


def test_noalloc_rejects_oversized_requests(lib):
    import torch
    from calcir_gb300._lib import CirError, check, load
    n, nmat = 1024, 8            # about 4.3 MiB of scratch per matrix: beyond the 8 MiB array
    dA = torch.zeros((nmat, n, n), dtype=torch.float32, device="cuda")
    dw = torch.zeros((nmat, n), dtype=torch.float32, device="cuda")
    with pytest.raises(CirError, match="scratch"):
        check(load().cir_eigh_noalloc(nmat, n, C.c_void_p(dA.data_ptr()), C.c_void_p(dw.data_ptr()), None))
    hA = np.zeros((1, 4, 4), np.float32)
    hw = np.zeros((1, 4), np.float32)
    with pytest.raises(CirError, match="device"):
        check(load().cir_eigh_noalloc(1, 4, C.c_void_p(hA.ctypes.data), C.c_void_p(hw.ctypes.data), None))
