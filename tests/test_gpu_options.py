"""The run options that reach the default run's results with less work.

share_frames: when time origins overlap (the full configuration places origins 2 ps apart,
each spanning 2.5 ps), each distinct frame is built and diagonalised once and counts in the
frequency distributions once per use.  propagate_vectors: the nine vectors psi_a = F m_a(0)
are propagated instead of F (O(N^2) per step instead of O(N^3)); the correlation functions
only ever contract F with m(0), so they are the same.  Both are exact rearrangements, so
both must reproduce the default run (and the FP64 oracle)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

KEYS = ("tcf_ir", "tcf_vv", "tcf_vh", "sw", "ls_ir", "ls_vv", "ls_vh")


def _prm(S=3, K=8):
    return {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0, "map": 0, "ntcfpoints": K,
            "nsamples": S, "sampleEvery": 0.03, "dt": 0.010, "t1": 0.260, "avef": 3415.0, "omegaStart": 1000,
            "omegaStop": 5000, "omegaStep": 1, "nzeros": 600, "beginTime": 0.0}


def _params(lib, prm, **extra):
    keys = {k: prm[k] for k in ("ntcfpoints", "nsamples", "sampleEvery", "omegaStep", "nchrom_mol", "nzeros",
                                "map", "dt", "t1", "avef", "beginTime", "omegaStart", "omegaStop")}
    keys.update(extra)
    return lib.default_params(model="tip4p2005", species="H2O", **keys)


def _run(lib, p, xyz, box, fos):
    with lib.Engine(p, xyz.shape[1]) as eng:
        out = eng.run(xyz, box, fos)
        return out, eng.stats()


def _same(a, b, tol, name):
    for k in KEYS:
        e = O.rel_l2(a[k], b[k])
        assert e < tol, (name, k, e)
    for k in ("pw", "rw", "rmw"):
        np.testing.assert_allclose(np.nan_to_num(a[k]), np.nan_to_num(b[k]), rtol=1e-6, atol=1e-9, err_msg=f"{name} {k}")
    assert a["bins_out_of_range"] == b["bins_out_of_range"], name


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_share_frames_reproduces_default(lib, precision):
    """3 origins 3 frames apart x 8 steps: 14 distinct frames instead of 24 eigensolves, the
    same correlation functions, spectra and (multiplicity-weighted) distributions."""
    prm = _prm()
    S, K = prm["nsamples"], prm["ntcfpoints"]
    fos = np.array([O.frame_index(prm, 0.010, s, k) for s in range(S) for k in range(K)], np.int32)
    nframes = int(fos.max()) + 1
    xyz, box = lib.synth_trajectory(40, nframes, seed=21)
    base, st0 = _run(lib, _params(lib, prm, precision=precision), xyz, box, fos)
    shared, st1 = _run(lib, _params(lib, prm, precision=precision, share_frames=1), xyz, box, fos)
    assert st0["eig_matrices"] == S * K
    assert st1["eig_matrices"] == len(np.unique(fos)) < S * K
    _same(shared, base, 1e-6, "shared " + precision)
    ref = O.run(prm, xyz, [box] * nframes, fos)
    for k in KEYS:
        assert O.rel_l2(shared[k], ref[k]) < (1e-4 if precision == "fp32" else 1e-3), k


def test_share_frames_irregular_origins_run_unshared(lib):
    """Origins that do not lie on one evenly spaced pattern are run without sharing."""
    prm = _prm(S=3, K=6)
    starts = [0, 2, 7]
    fos = np.array([s0 + k for s0 in starts for k in range(6)], np.int32)
    xyz, box = lib.synth_trajectory(32, int(fos.max()) + 1, seed=22)
    base, _ = _run(lib, _params(lib, prm), xyz, box, fos)
    shared, st = _run(lib, _params(lib, prm, share_frames=1), xyz, box, fos)
    assert st["eig_matrices"] == 18
    _same(shared, base, 1e-6, "irregular")


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_propagate_vectors_reproduces_default(lib, precision):
    """psi propagation against the F propagation of the same run and against the oracle; with
    frame sharing on as well."""
    prm = _prm()
    S, K = prm["nsamples"], prm["ntcfpoints"]
    fos = np.array([O.frame_index(prm, 0.010, s, k) for s in range(S) for k in range(K)], np.int32)
    nframes = int(fos.max()) + 1
    xyz, box = lib.synth_trajectory(40, nframes, seed=23)
    full, _ = _run(lib, _params(lib, prm, precision=precision), xyz, box, fos)
    vec, st = _run(lib, _params(lib, prm, precision=precision, propagate_vectors=1), xyz, box, fos)
    both, st2 = _run(lib, _params(lib, prm, precision=precision, propagate_vectors=1, share_frames=1), xyz, box, fos)
    tol = 1e-5 if precision == "fp32" else 1e-3
    _same(vec, full, tol, "vectors " + precision)
    _same(both, vec, 1e-6, "vectors + shared " + precision)
    assert st2["eig_matrices"] < st["eig_matrices"]
    ref = O.run(prm, xyz, [box] * nframes, fos)
    for k in KEYS:
        assert O.rel_l2(vec[k], ref[k]) < (1e-4 if precision == "fp32" else 1e-3), k
