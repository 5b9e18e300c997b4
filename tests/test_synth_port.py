"""The CPU legs of bench.py (no GPU): the numpy restatement of the seeded frame generator
(oracle/synth.py) reproduces the library's generator bit for bit, and the CPU timing port
of the reference algorithm (oracle/cpu_reference.py) builds the same Hamiltonian as the
FP64 oracle and runs one frame-step."""
import numpy as np
import pytest

from oracle import cpu_reference as R
from oracle import oracle as O
from oracle import synth


@pytest.mark.parametrize("nmol,nframes,seed", [(64, 40, 11), (216, 25, 5), (512, 16, 1), (1024, 4, 2)])
def test_numpy_generator_is_bit_identical(lib, nmol, nframes, seed):
    a, box_a = lib.synth_trajectory(nmol, nframes, seed=seed)
    b, box_b = synth.trajectory(nmol, nframes, seed=seed)
    assert np.array_equal(box_a, box_b)
    assert np.array_equal(a, b)


def test_numpy_generator_contacts():
    """No O/H contact below 0.15 nm between molecules, as the generator promises."""
    xyz, box = synth.trajectory(64, 10, seed=3)
    L = float(box[0])
    for f in range(10):
        m = xyz[f].reshape(64, 4, 3)[:, :3].astype(np.float64)
        d = m[:, None, :, None, :] - m[None, :, None, :, :]
        d -= L * np.round(d / L)
        r = np.sqrt((d * d).sum(-1))
        r[np.arange(64), np.arange(64)] = 1.0
        assert r.min() >= 0.15 - 1e-6


def test_cpu_port_build_matches_oracle(lib):
    xyz, box = lib.synth_trajectory(128, 2, seed=4)
    prm = {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0, "map": 0, "avef": 3415.0, "dt": 0.01}
    E, H, dip, pol = O.frame(xyz[1], box, prm)
    H32, m = R.build(xyz[1], box, prm)
    assert np.abs(H32 - H).max() <= 1e-5 * np.abs(H).max()
    np.testing.assert_allclose(m, np.vstack([dip, pol]), rtol=1e-5, atol=1e-7)
    # one frame-step at k = 0 and k = 1: F = I, then one propagator product
    state = {}
    t0 = R.frame_step(xyz[0], box, prm, state)
    t1 = R.frame_step(xyz[1], box, prm, state)
    assert len(t0) == len(t1) == 15
    F = state["F"]
    assert np.abs(F.conj().T @ F - np.eye(F.shape[0])).max() < 1e-4
