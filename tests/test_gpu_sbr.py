"""The two-stage reduction to tridiagonal form (cir_tridiag_sbr: dense -> band on the
split-BF16 tcgen05 GEMM, band -> tridiagonal by bulge chasing) against FP64 eigenvalues."""
import numpy as np
import pytest
from scipy.linalg import eigvalsh_tridiagonal

import calcir_gb300 as cg
from calcir_gb300._lib import CirError

pytestmark = pytest.mark.gpu


def _tridiag_eigs(d, e):
    return np.stack([eigvalsh_tridiagonal(d[i].astype(np.float64), e[i, :-1].astype(np.float64))
                     for i in range(d.shape[0])])


def _errs(A, d, e):
    w64 = np.linalg.eigvalsh(A.astype(np.float64))
    w = _tridiag_eigs(d, e)
    spread = w64[:, -1] - w64[:, 0]
    return np.abs(w - w64).max(axis=1) / spread


@pytest.mark.parametrize("n", [3, 33, 64, 67, 130, 300, 515])
def test_sbr_random_symmetric(n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((3, n, n)).astype(np.float32)
    A = (a + np.swapaxes(a, 1, 2)) * np.float32(0.5) + np.float32(3.0) * np.eye(n, dtype=np.float32)
    with cg.Engine(cg.default_params(species="H2O"), 8) as eng:
        d, e, ms = eng.tridiag_sbr(A)
    err = _errs(A, d, e)
    print(f"n={n}: eigenvalue error / spread {err.max():.2e}, stages {ms[0]:.2f} / {ms[1]:.2f} ms")
    assert np.all(err < 2e-4), err


def test_sbr_water_hamiltonians_order_1024():
    xyz, box = cg.synth_trajectory(512, 4, seed=3)
    p = cg.default_params(model="tip4p2005", species="H2O", avef=3415.0)
    with cg.Engine(p, xyz.shape[1]) as eng:
        H, _, _, _ = eng.build_hamiltonian(xyz, box)
        d, e, ms = eng.tridiag_sbr(H)
    w64 = np.linalg.eigvalsh(H.astype(np.float64))
    w = _tridiag_eigs(d, e)
    err_abs = np.abs(w - w64).max()
    spread = (w64[:, -1] - w64[:, 0]).min()
    print(f"order 1024 water: max |dw| {err_abs:.3e} cm-1 (spread {spread:.0f} cm-1), stages {ms[0]:.2f} / {ms[1]:.2f} ms")
    assert err_abs / spread < 5e-5


def test_sbr_rejects_orders_above_its_schedule():
    with cg.Engine(cg.default_params(species="H2O"), 8) as eng:
        with pytest.raises(CirError, match="exceeds"):
            eng.tridiag_sbr(np.eye(1100, dtype=np.float32)[None])
