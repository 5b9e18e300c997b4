"""The differentiation form on the GPU: cir_loss_grad (the adjoint of the propagation and
the eigendecompositions, through the maps) against FP64 references of the same loss --
central finite differences and the numpy adjoint of oracle/adjoint.py.  Gradients are
compared as theta_i dL/dtheta_i (the loss's sensitivity to a relative change of each
coefficient), whose components are comparable in size; the bar is 1e-3 of the largest."""
import numpy as np
import pytest

from oracle import adjoint as A
from oracle import oracle as O

pytestmark = pytest.mark.gpu

BAR = 1e-3


def _setup(lib, nmol, S, K, nzeros, seed=4):
    prm = {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0, "map": 0, "ntcfpoints": K,
           "nsamples": S, "sampleEvery": 0.03, "dt": 0.010, "t1": 0.260, "avef": 3415.0, "omegaStart": 2000,
           "omegaStop": 5000, "omegaStep": 1, "nzeros": nzeros, "beginTime": 0.0}
    nframes = 3 * (S - 1) + K
    xyz, box = lib.synth_trajectory(nmol, nframes, seed=seed)
    fos = np.array([O.frame_index(prm, 0.010, s, k) for s in range(S) for k in range(K)], np.int32)
    th0 = A.theta_of(O.maps(0, 0))
    tht = (th0 * (1 + 0.02 * np.random.default_rng(1).uniform(-1, 1, 13))).astype(np.float32).astype(np.float64)
    tir, tvv, _ = A.forward(prm, tht, xyz, [box] * nframes, fos)
    targets = [t.astype(np.float32) for t in A.lineshapes(prm, tir, tvv)]
    p = lib.default_params(model="tip4p2005", species="H2O", map=0, ntcfpoints=K, nsamples=S, sampleEvery=0.03,
                           dt=0.010, t1=0.260, avef=3415.0, omegaStart=2000, omegaStop=5000, omegaStep=1,
                           nzeros=nzeros)
    return prm, p, xyz, box, fos, th0, targets


def _close(g, ref, th, name):
    s, sr = g * th, ref * th
    scale = np.abs(sr).max()
    err = np.abs(s - sr) / scale
    assert err.max() <= BAR, (name, err.max(), list(zip(A.THETA_NAMES, err)))
    return err.max()


def test_loss_grad_against_central_differences(lib):
    """16 molecules, 2 origins x 6 steps: loss and gradient against FP64 central differences."""
    prm, p, xyz, box, fos, th0, targets = _setup(lib, 16, 2, 6, 300)
    with lib.Engine(p, xyz.shape[1]) as eng:
        np.testing.assert_array_equal(eng.get_coeffs(), th0.astype(np.float32))
        L, g = eng.loss_grad(xyz, box, fos, targets[0], targets[1])
    boxes = [box] * len(xyz)
    t64 = [t.astype(np.float64) for t in targets]
    Lref = A.loss(prm, th0, xyz, boxes, fos, t64)
    assert abs(L - Lref) <= BAR * Lref, (L, Lref)
    gfd = A.fd_grad(prm, th0, xyz, boxes, fos, t64)
    _close(g, gfd, th0, "central differences")


def test_loss_grad_across_checkpoint_segments(lib):
    """24 molecules, 2 origins x 40 steps (three checkpoint segments of 16 steps) against the
    FP64 adjoint."""
    prm, p, xyz, box, fos, th0, targets = _setup(lib, 24, 2, 40, 400, seed=7)
    with lib.Engine(p, xyz.shape[1]) as eng:
        L, g = eng.loss_grad(xyz, box, fos, targets[0], targets[1])
    Lref, gref = A.adjoint_grad(prm, th0, xyz, [box] * len(xyz), fos, [t.astype(np.float64) for t in targets])
    assert abs(L - Lref) <= BAR * Lref, (L, Lref)
    _close(g, gref, th0, "FP64 adjoint")


def test_autograd_wrapper_and_gpu_central_difference(lib):
    """torch.autograd through the C-ABI backward gives the library's gradient, and a GPU
    central difference (relative step 1e-4) of the most sensitive coefficient agrees."""
    import torch
    from calcir_gb300.autograd import SpectrumLoss
    prm, p, xyz, box, fos, th0, targets = _setup(lib, 16, 2, 6, 300)
    with lib.Engine(p, xyz.shape[1]) as eng:
        theta = torch.tensor(th0.astype(np.float32).astype(np.float64), requires_grad=True)
        loss = SpectrumLoss.apply(theta, eng, xyz, box, fos, targets[0], targets[1])
        loss.backward()
        eng.set_coeffs(th0.astype(np.float32))
        L, g = eng.loss_grad(xyz, box, fos, targets[0], targets[1])
        np.testing.assert_allclose(theta.grad.numpy(), g, rtol=1e-12)
        assert float(loss.detach()) == pytest.approx(L, rel=1e-12)
        q = int(np.argmax(np.abs(g * th0)))
        h = 1e-4 * abs(th0[q])
        vals = []
        for sgn in (1, -1):
            t = th0.copy()
            t[q] += sgn * h
            eng.set_coeffs(t.astype(np.float32))
            vals.append(eng.loss_grad(xyz, box, fos, targets[0], targets[1])[0])
        hq = float(np.float32(th0[q] + h)) - float(np.float32(th0[q] - h))   # the step as stored in float32
        fd = (vals[0] - vals[1]) / hq
        assert abs(fd - g[q]) <= 2e-2 * abs(g[q]), (A.THETA_NAMES[q], fd, g[q])


def test_loss_grad_config_size(lib):
    """The differentiation configuration itself -- 256 molecules (512 chromophores), 4 origins
    x 200 points, targets from map coefficients perturbed by seeded +-2% noise -- against the
    loss and the FP64 adjoint gradient stored by tests/golden/make_configs.py."""
    import os
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import make_configs as MC
    path = os.path.join(GOLDEN, "diff_256h2o.npz")
    if not os.path.exists(path):
        pytest.skip("diff_256h2o.npz not generated (tests/golden/make_configs.py)")
    z = np.load(path)
    xyz, box, fos = MC.diff_frames(lib.synth_trajectory)
    assert np.array_equal(fos, z["frame_table"])
    q = {k: MC.DIFF_PRM[k] for k in ("ntcfpoints", "nsamples", "sampleEvery", "omegaStep", "nzeros", "map", "dt",
                                     "t1", "avef", "beginTime", "omegaStart", "omegaStop")}
    p = lib.default_params(model="tip4p2005", species="H2O", **q)
    th0 = z["theta0"]
    with lib.Engine(p, xyz.shape[1]) as eng:
        np.testing.assert_array_equal(eng.get_coeffs(), th0.astype(np.float32))
        L, g = eng.loss_grad(xyz, box, fos.astype(np.int32), z["target_ir"], z["target_vv"])
    Lref = float(z["loss"])
    assert abs(L - Lref) <= BAR * Lref, (L, Lref)
    err = _close(g, z["grad"], th0, "FP64 adjoint, 256 H2O 4 x 200")
    print(f"config-size gradient: worst theta_i dL/dtheta_i error {err:.2e} of the largest")
