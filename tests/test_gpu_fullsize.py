"""Full-length parity of the two large configurations against the FP64 oracle.

The oracle's whole job (FP64, psi-vector propagation) was run once on each configuration's
seeded frames and stored as a fixture (tests/golden/make_fullsize.py):

  512 molecules (1024 chromophores), 10 time origins 2 ps apart x 250 points -- the timed
  job of bench.py, frames of seed 1
  1024 molecules (2048 chromophores), 5 origins x 250 points, frames of seed 1

Every form runs the same job through the C ABI (cir_run) and is held to the bound its form
states, per spectrum (IR, VV, VH correlation functions and lineshapes, spectral density):
the plain FP32 form within 1e-4 relative L2, the mixed forms (split-BF16 and TF32 tensor-core
GEMMs, with and without the FP64 eigenpair refinement, and the split-BF16 form with frame
sharing or the psi-vector propagation) within 1e-3.  The frequency
distributions agree up to bin flips of eigenvalues that sit on a bin edge.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle as O

sys.path.insert(0, GOLDEN)
import make_fullsize as MF  # noqa: E402

pytestmark = pytest.mark.gpu

SPEC_TOL = 1e-4
MIXED_TOL = 1e-3
KEYS = ("tcf_ir", "tcf_vv", "tcf_vh", "ls_ir", "ls_vv", "ls_vh", "sw")

_CACHE = {}


def _case(lib, nmol):
    """(oracle parameters, oracle result, positions, box, frame table) of a fixture."""
    if nmol not in _CACHE:
        path = os.path.join(GOLDEN, MF.CONFIGS[nmol]["name"] + ".npz")
        if not os.path.exists(path):
            pytest.skip(f"{path} not generated (tests/golden/make_fullsize.py)")
        prm, acc, nm, seed, fos = MF.load(path)
        ref = O.finish(prm, acc)
        xyz, box = lib.synth_trajectory(nm, int(fos.max()) + 1, seed=seed)
        _CACHE[nmol] = (prm, ref, xyz, box, np.asarray(fos, np.int32))
    return _CACHE[nmol]


def _params(lib, prm, **extra):
    keys = {k: prm[k] for k in ("ntcfpoints", "nsamples", "sampleEvery", "omegaStep", "nzeros", "map", "dt", "t1",
                                "avef", "beginTime", "omegaStart", "omegaStop")}
    keys.update(extra)
    return lib.default_params(model="tip4p2005", species="H2O", **keys)


# the options of the same job (distinct frames diagonalised once; psi = F m(0) propagated)
# run the split eigensolver's two streams with the frame weights and the vector propagation
FORMS = [("fp32", {}), ("bf16x3", {}), ("tf32", {}), ("bf16x3+refine2", {"refine_eigen": 2}),
         ("bf16x3+share", {"share_frames": 1}), ("bf16x3+vectors", {"propagate_vectors": 1})]


@pytest.mark.parametrize("nmol", [512, 1024])
@pytest.mark.parametrize("form", [f for f, _ in FORMS])
def test_full_length_against_oracle(lib, nmol, form):
    prm, ref, xyz, box, fos = _case(lib, nmol)
    precision = form.split("+")[0]
    extra = dict(FORMS)[form]
    # the frame table the library computes (calcIR.cu:378-379 in float) is the oracle's
    p = _params(lib, prm, precision=precision, **extra)
    assert np.array_equal(lib.frame_table(p, MF.FRAME_DT), fos)
    with lib.Engine(p, xyz.shape[1]) as eng:
        out = eng.run(xyz, box, fos)
        st = eng.stats()
    assert st["frame_steps"] == len(fos)
    errs = {k: O.rel_l2(out[k], ref[k]) for k in KEYS}
    # per-step error of the correlation functions (relative to each function's t = 0 value)
    step_err = max(float(np.max(np.abs(out[k] - ref[k])) / np.abs(ref[k][0])) for k in ("tcf_ir", "tcf_vv", "tcf_vh"))
    print(f"{nmol} H2O {prm['nsamples']}x{prm['ntcfpoints']} {form}:",
          {k: f"{v:.2e}" for k, v in errs.items()}, f"max per-step {step_err:.2e}")
    tol = SPEC_TOL if form == "fp32" else MIXED_TOL
    for k, v in errs.items():
        assert v < tol, (k, v)
    np.testing.assert_array_equal(out["ls_omega"], np.asarray(ref["ls_omega"], np.float32))
    assert out["bins_out_of_range"] == ref["bins_out_of_range"]
    ntot = np.sum(ref["count"])
    step = prm["omegaStep"]
    assert np.max(np.abs(np.cumsum(out["pw"]) - np.cumsum(ref["pw"]))) * step <= 16.0 / ntot + 1e-6
    for k in ("rw", "rmw"):
        a, b = np.nan_to_num(out[k] * out["pw"]), np.nan_to_num(ref[k] * ref["pw"])
        assert np.max(np.abs(np.cumsum(a) - np.cumsum(b))) <= 16.0 * np.abs(b).max() + 1e-6 * np.abs(b).sum()
