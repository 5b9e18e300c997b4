"""Pins the FP64 oracle against golden outputs of the reference program itself.

The fixtures in tests/golden were written by the reference's own calcIR.cu built for the
host (oracle/build_ref.sh, tests/golden/make_golden.py) on seeded synthetic trajectories.
The reference runs in FP32; the oracle in FP64; spectra agree within 1e-4 relative L2."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, golden_params, load_golden
from oracle import oracle as O

TOL = 1e-4   # relative L2 per spectrum, FP32 reference vs FP64 oracle


def run_oracle(lib, meta):
    prm = golden_params(meta)
    xyz, box = lib.synth_trajectory(meta["nmol"], meta["nframes"], seed=meta["seed"])
    fos = [O.frame_index(prm, meta["frame_dt"], s, k)
           for s in range(prm["nsamples"]) for k in range(prm["ntcfpoints"])]
    return prm, O.run(prm, xyz, [box] * len(xyz), fos)


@pytest.fixture(scope="module", params=GOLDEN_CASES)
def case(request, lib):
    meta, gold = load_golden(request.param)
    prm, out = run_oracle(lib, meta)
    return request.param, prm, out, gold


def test_tcf(case):
    name, prm, out, gold = case
    K = prm["ntcfpoints"]
    t = np.arange(K) * np.float32(prm["dt"])
    for key, f in (("tcf_ir", "ir"), ("tcf_vv", "vv"), ("tcf_vh", "vh")):
        ref = gold[f + "rtcf"][:, 1] + 1j * gold[f + "itcf"][:, 1]
        np.testing.assert_array_equal(gold[f + "rtcf"][:, 0], O.as_printed(t))
        assert O.rel_l2(out[key], ref) < TOL, (name, key, O.rel_l2(out[key], ref))


def test_spectral_density(case):
    name, prm, out, gold = case
    np.testing.assert_array_equal(gold["spdn"][:, 0], O.as_printed(out["omega"]))
    assert O.rel_l2(out["sw"], gold["spdn"][:, 1]) < TOL


def test_lineshapes(case):
    name, prm, out, gold = case
    for key, f in (("ls_ir", "irls"), ("ls_vv", "vvls"), ("ls_vh", "vhls")):
        assert gold[f].shape[0] == len(out["ls_omega"]), (name, f)
        np.testing.assert_array_equal(gold[f][:, 0], O.as_printed(out["ls_omega"]))
        assert O.rel_l2(out[key], gold[f][:, 1]) < TOL, (name, key, O.rel_l2(out[key], gold[f][:, 1]))


def test_frequency_distributions(case):
    """Pw/Rw/Rmw are histograms of eigenvalues: FP32 and FP64 eigenvalues may fall in
    neighbouring bins, so compare cumulative sums (a flip moves mass by one bin)."""
    name, prm, out, gold = case
    step = prm["omegaStep"]
    pw_ref, pw = gold["Pw"][:, 1], out["pw"]
    assert abs(pw.sum() * step - 1.0) < 1e-9
    assert abs(pw_ref.sum() * step - 1.0) < 1e-5
    ntot = out["count"].sum()
    assert np.max(np.abs(np.cumsum(pw) - np.cumsum(pw_ref))) * step <= 4.0 / ntot + 1e-6
    for key, f in (("rw", "Rw"), ("rmw", "Rmw")):
        a = np.nan_to_num(out[key] * pw)
        b = np.nan_to_num(gold[f][:, 1] * pw_ref)
        scale = np.abs(b).sum()
        assert np.max(np.abs(np.cumsum(a) - np.cumsum(b))) <= 4.0 * np.abs(b).max() + 1e-6 * scale
        # NaN exactly where the histogram is empty (calcIR.cu:836-839)
        both = (out["count"] > 0) == (pw_ref > 0)
        assert np.mean(both) > 0.995


@pytest.mark.parametrize("name", ["fullsize_512h2o", "fullsize_1024h2o"])
def test_fullsize_fixture_finished_spectra(name):
    """The finished spectra stored beside the raw sums of a full-length fixture (bench.py
    reads them to state the error of its timed run) are what the oracle makes of the sums."""
    import sys
    sys.path.insert(0, GOLDEN)
    import make_fullsize as MF
    path = os.path.join(GOLDEN, name + ".npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    prm, acc, _, _, fos = MF.load(path)
    assert len(fos) == prm["nsamples"] * prm["ntcfpoints"]
    fin = O.finish(prm, acc)
    z = np.load(path)
    for k in ("tcf_ir", "tcf_vv", "tcf_vh", "sw", "ls_ir", "ls_vv", "ls_vh"):
        assert O.rel_l2(z["fin_" + k], fin[k]) < 1e-7, k
    assert int(z["fin_ls_len"]) == len(fin["ls_omega"])
