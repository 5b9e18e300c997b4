"""Failure detection on the GPU path, driven without faulting or hanging the GPU.

The reference stops the process on any error (calcIR.h:44-46; magma_ssyevd's info,
calcIR.cu:445).  Here every wait of the tensor-core pipeline is bounded and the eigensolver
caps its iterations; both turn into an error status the host reads.  Two fault drills of
cir_params (off by default) make them fire on purpose:

  test_stall_gemm  the persistent split-BF16 GEMM withholds its first tile's completion
                   signal, a flag nothing else sets; its shortened bounded waits run out, every
                   role leaves its loop after its copies and MMAs in flight have completed, and
                   the call returns CIR_ERR_CUDA ("timed out")
  test_sweep_cap   the divide-and-conquer leaves may take one QR sweep, which they cannot
                   converge in; cir_eigh returns CIR_ERR_NOCONVERGE

After each failure the same process runs a normal call on a fresh context and gets correct
results: the CUDA context stays usable.
"""
import numpy as np
import pytest

from calcir_gb300._lib import CirError

pytestmark = pytest.mark.gpu

ERR_CUDA, ERR_NOCONVERGE = -2, -4


def _sym(rng, n, scale=1000.0):
    a = rng.standard_normal((n, n))
    return ((a + a.T) * (scale / np.sqrt(8 * n))).astype(np.float32)


def _normal_eigh_works(lib, A, precision):
    with lib.Engine(lib.default_params(species="H2O", precision=precision), 8) as eng:
        w, V = eng.eigh(A)
    for m in range(A.shape[0]):
        wref = np.linalg.eigvalsh(A[m].astype(np.float64))
        assert np.abs(w[m] - wref).max() <= 2e-5 * np.abs(wref).max()


def test_gemm_pipeline_stall_is_reported(lib):
    """The eigensolver's split-BF16 back-transform (k_tc_persist) under the stall drill."""
    rng = np.random.default_rng(3)
    A = np.stack([_sym(rng, 256) for _ in range(4)])
    with lib.Engine(lib.default_params(species="H2O", precision="bf16x3", test_stall_gemm=1), 8) as eng:
        with pytest.raises(CirError, match="timed out") as ei:
            eng.eigh(A)
        assert ei.value.code == ERR_CUDA
        # the same context reports the drill again on the next call, without a GPU error
        with pytest.raises(CirError, match="timed out"):
            eng.eigh(A)
    _normal_eigh_works(lib, A, "bf16x3")


def test_gemm_pipeline_stall_in_a_run(lib):
    """A whole job in the split-BF16 form (propagation and back-transform on k_tc_persist)."""
    xyz, box = lib.synth_trajectory(64, 6, seed=2)
    p = lib.default_params(model="tip4p2005", species="H2O", ntcfpoints=6, nsamples=1, omegaStep=2, nzeros=200,
                           omegaStart=1000, omegaStop=5000, precision="bf16x3", test_stall_gemm=1)
    with lib.Engine(p, xyz.shape[1]) as eng:
        with pytest.raises(CirError, match="timed out"):
            eng.run(xyz, box)
    p.test_stall_gemm = 0
    with lib.Engine(p, xyz.shape[1]) as eng:
        out = eng.run(xyz, box)
    assert np.all(np.isfinite(out["tcf_ir"])) and abs(out["tcf_ir"][0]) > 0


def test_eigensolver_sweep_cap_is_reported(lib):
    rng = np.random.default_rng(5)
    A = np.stack([_sym(rng, 300) for _ in range(3)])
    for precision in ("fp32", "bf16x3"):
        with lib.Engine(lib.default_params(species="H2O", precision=precision, test_sweep_cap=1), 8) as eng:
            with pytest.raises(CirError, match="sweep cap") as ei:
                eng.eigh(A)
            assert ei.value.code == ERR_NOCONVERGE
        _normal_eigh_works(lib, A, precision)
