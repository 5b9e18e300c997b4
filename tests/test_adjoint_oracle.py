"""The FP64 reference of the differentiation form: the adjoint gradient of the
spectrum-mismatch loss (oracle/adjoint.py, the algorithm the CUDA path implements) against
central finite differences of the FP64 forward, on a small seeded system whose target
lineshapes come from map coefficients perturbed by seeded +-2% noise."""
import numpy as np

import calcir_gb300 as cg
from oracle import adjoint as A
from oracle import oracle as O


def _case():
    prm = {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0, "map": 0, "ntcfpoints": 6,
           "nsamples": 2, "sampleEvery": 0.03, "dt": 0.010, "t1": 0.260, "avef": 3415.0, "omegaStart": 2000,
           "omegaStop": 5000, "omegaStep": 1, "nzeros": 300, "beginTime": 0.0}
    xyz, box = cg.synth_trajectory(16, 12, seed=4)
    fos = [O.frame_index(prm, 0.010, s, k) for s in range(2) for k in range(6)]
    th0 = A.theta_of(O.maps(0, 0))
    tht = th0 * (1 + 0.02 * np.random.default_rng(1).uniform(-1, 1, 13))
    tir, tvv, _ = A.forward(prm, tht, xyz, [box] * len(xyz), fos)
    return prm, xyz, [box] * len(xyz), fos, th0, A.lineshapes(prm, tir, tvv)


def test_adjoint_matches_central_differences():
    prm, xyz, boxes, fos, th0, targets = _case()
    L, g = A.adjoint_grad(prm, th0, xyz, boxes, fos, targets)
    gfd = A.fd_grad(prm, th0, xyz, boxes, fos, targets)
    assert L > 0
    np.testing.assert_allclose(g, gfd, rtol=1e-5, atol=0)


def test_loss_vanishes_at_the_target_coefficients():
    prm, xyz, boxes, fos, th0, _ = _case()
    tir, tvv, _ = A.forward(prm, th0, xyz, boxes, fos)
    targets = A.lineshapes(prm, tir, tvv)
    L, g = A.adjoint_grad(prm, th0, xyz, boxes, fos, targets)
    assert L == 0 and np.all(g == 0)
