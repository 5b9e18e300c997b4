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


def _device_copy(A, offset_bytes=0):
    """A device copy of A whose first element sits offset_bytes past a 256-byte boundary."""
    import torch
    nmat, n = A.shape[0], A.shape[-1]
    pad = offset_bytes // 4
    flat = torch.zeros(nmat * n * n + pad, dtype=torch.float32, device="cuda")
    dA = flat[pad:].view(nmat, n, n)
    dA.copy_(torch.from_numpy(np.ascontiguousarray(A)))
    return flat, dA


def _call(dA, dw):
    from calcir_gb300._lib import check, load
    nmat, n = dA.shape[0], dA.shape[-1]
    check(load().cir_eigh_noalloc(nmat, n, C.c_void_p(dA.data_ptr()), C.c_void_p(dw.data_ptr()), None))


def _noalloc(A, offset_bytes=0):
    """cir_eigh_noalloc through the C ABI on a device copy of A; returns (w, V) on the host."""
    import torch
    nmat, n = A.shape[0], A.shape[-1]
    keep, dA = _device_copy(A, offset_bytes)
    assert dA.data_ptr() % 16 == offset_bytes % 16
    dw = torch.empty((nmat, n), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    _call(dA, dw)
    V = np.ascontiguousarray(np.swapaxes(dA.cpu().numpy(), 1, 2))   # column j = eigenvector j
    return dw.cpu().numpy(), V


def _check(A, w0, V0, w1, tag):
    """Eigenvalues against FP64 LAPACK and cir_eigh's; eigenpairs reproduce A; orthogonality."""
    n = A.shape[0]
    wref = np.linalg.eigvalsh(A.astype(np.float64))
    nrm = np.abs(wref).max()
    scale = max(1.0, np.sqrt(n) / 4)
    assert np.abs(w0 - wref).max() <= 2e-6 * nrm * scale, tag
    assert np.abs(w0 - w1).max() <= 2e-6 * nrm * scale, tag
    R0 = (V0.astype(np.float64) * w0) @ V0.T.astype(np.float64)
    assert np.abs(R0 - A).max() <= 4e-6 * nrm * scale, tag
    assert np.abs(V0.T.astype(np.float64) @ V0 - np.eye(n)).max() <= 2e-6 * max(1.0, np.sqrt(n)), tag


@pytest.mark.parametrize("n,nmat,offset", [(130, 3, 0), (256, 2, 0), (200, 2, 4), (512, 7, 0), (1024, 1, 0)])
def test_noalloc_matches_cir_eigh_twice(lib, n, nmat, offset):
    """Two calls in a row agree with cir_eigh (the allocating entry point) and with FP64
    eigvalsh within the eigensolver tolerance the other tests use; covers an order that is
    not a multiple of 4 (130), an A 4 bytes off 16-byte alignment (200), and the documented
    batch limits (7 of order 512, 1 of order 1024)."""
    rng = np.random.default_rng(n + offset)
    for call in range(2):
        A = np.stack([_sym(rng, n) for _ in range(nmat)])
        w0, V0 = _noalloc(A, offset)
        with lib.Engine(lib.default_params(species="H2O"), 8) as eng:
            w1, _ = eng.eigh(A)
        for m in range(nmat):
            _check(A[m], w0[m], V0[m], w1[m], (call, m))


def test_noalloc_allocates_nothing(lib):
    """After a warm-up call, a call leaves the device's free memory unchanged."""
    import torch
    rng = np.random.default_rng(7)
    A = np.stack([_sym(rng, 256) for _ in range(4)])
    _, dA = _device_copy(A)
    dw = torch.empty((4, 256), dtype=torch.float32, device="cuda")
    _call(dA, dw)                                 # warm-up: symbol lookup, module load
    dA.copy_(torch.from_numpy(A))
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    _call(dA, dw)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    w = dw.cpu().numpy()
    for m in range(4):
        assert np.abs(w[m] - np.linalg.eigvalsh(A[m].astype(np.float64))).max() <= 2e-6 * 1000 * 4


def test_noalloc_rejects_oversized_requests(lib):
    import torch
    from calcir_gb300._lib import CirError, check, load
    n, nmat = 1024, 8            # about 4.3 MiB of scratch per matrix: beyond the 8 MiB array
    dA = torch.zeros((nmat, n, n), dtype=torch.float32, device="cuda")
    dw = torch.zeros((nmat, n), dtype=torch.float32, device="cuda")
    with pytest.raises(CirError, match="fewer matrices"):
        check(load().cir_eigh_noalloc(nmat, n, C.c_void_p(dA.data_ptr()), C.c_void_p(dw.data_ptr()), None))
    n = 1500                     # one matrix of this order does not fit: the message names the limit
    dA = torch.zeros((1, n, n), dtype=torch.float32, device="cuda")
    dw = torch.zeros((1, n), dtype=torch.float32, device="cuda")
    with pytest.raises(CirError, match="orders up to 1412"):
        check(load().cir_eigh_noalloc(1, n, C.c_void_p(dA.data_ptr()), C.c_void_p(dw.data_ptr()), None))
    hA = np.zeros((1, 4, 4), np.float32)
    hw = np.zeros((1, 4), np.float32)
    with pytest.raises(CirError, match="device"):
        check(load().cir_eigh_noalloc(1, 4, C.c_void_p(hA.ctypes.data), C.c_void_p(hw.ctypes.data), None))
