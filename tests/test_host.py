"""Host-side logic of the drop-in boundary (no GPU): parser, defaults, sizes, frame
indexing, trajectory files, the synthetic generator, output formats and the C ABI."""
import ctypes as C
import hashlib
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, GOLDEN_CASES, ROOT, golden_params, load_golden
from oracle import oracle as O


def test_abi_exports_every_declared_symbol(lib):
    """libcalcir.so loads and exports every function include/calcir.h declares."""
    src = open(os.path.join(ROOT, "include", "calcir.h")).read()
    declared = set(re.findall(r"^(?:const char \*|int )\s*(cir_\w+)\s*\(", src, re.M))
    assert len(declared) >= 25
    dll = C.CDLL(lib.LIB_PATH)
    missing = [s for s in declared if not hasattr(dll, s)]
    assert not missing, missing
    from calcir_gb300._lib import SIGNATURES
    assert declared == set(SIGNATURES), declared ^ set(SIGNATURES)


def test_defaults_match_reference(lib):
    p = lib.default_params()   # calcIR.cu:36-59
    assert (p.ntcfpoints, p.nsamples, p.omegaStep, p.natom_mol, p.nchrom_mol, p.nzeros, p.map) == \
        (150, 1, 5, 4, 2, 25600, 0)
    assert p.xtcf == b"traj.xtc" and p.outf == b"spec" and p.model == b"e3b3" and p.species == b" "
    assert np.float32(p.sampleEvery) == np.float32(10.0) and np.float32(p.dt) == np.float32(0.010)
    assert np.float32(p.t1) == np.float32(0.260) and np.float32(p.avef) == np.float32(3415.2)
    assert (p.omegaStart, p.omegaStop, p.beginTime) == (2000.0, 5000.0, 0.0)


def _printed(p):
    """The parameter lines the reference prints after parsing (calcIR.cu:70-87)."""
    d = lambda s: s.decode()
    return [f"\tSetting xtc file {d(p.xtcf)}", f"\tSetting default file name to {d(p.outf)}",
            f"\tSetting model to {d(p.model)}", f"\tSetting the number of tcf points to {p.ntcfpoints}",
            f"\tSetting nsamples to {p.nsamples}", "\tSetting sampleEvery to %f (ps)" % p.sampleEvery,
            f"\tSetting omegaStep to {p.omegaStep}", f"\tSetting natom_mol to {p.natom_mol}",
            f"\tSetting nchrom_mol to {p.nchrom_mol}", f"\tSetting nzeros to {p.nzeros}",
            f"\tSetting map to {p.map}", f"\tSetting species to {d(p.species)}",
            "\tSetting omegaStart to %f" % p.omegaStart, "\tSetting omegaStop to %f" % p.omegaStop,
            "\tSetting dt to %f" % p.dt, "\tSetting t1 to %f (ps)" % p.t1, "\tSetting avef to %f" % p.avef,
            "\tSetting equilibration time to %f (ps)" % p.beginTime]


@pytest.mark.parametrize("case", ["parse_basic", "parse_quirks"])
def test_parser_matches_reference(lib, case, tmp_path, capfd):
    """cir_params_parse_file reproduces the values the reference's ir_init parses from the
    same file (golden: the reference's own printout), including its token quirks."""
    g = json.load(open(os.path.join(GOLDEN, case + ".json")))
    f = tmp_path / "input.inp"
    f.write_text(g["input"])
    p = lib.parse_input(str(f))
    ref_settings = [ln for ln in g["stdout"] if ln.startswith("\tSetting")]
    assert _printed(p) == ref_settings
    out = capfd.readouterr().out
    ref_warn = [ln.replace("input.inp", str(f)) for ln in g["stdout"] if "not recognized" in ln]
    assert [ln for ln in out.splitlines() if "not recognized" in ln] == ref_warn


def test_finalize_rejects_what_the_reference_aborts_on(lib):
    from calcir_gb300 import CirError, finalize
    with pytest.raises(CirError, match="species"):
        finalize(lib.default_params())                    # default species " " aborts (calcIR.cu:336-339)
    with pytest.raises(CirError, match="model"):
        finalize(lib.default_params(species="H2O", model="spc"))
    with pytest.raises(CirError, match="map"):
        finalize(lib.default_params(species="H2O", map=2))
    p = finalize(lib.default_params(species="HOD/H2O", model="tip4p"))
    assert (p.imodel, p.ispecies) == (0, 2)
    p = finalize(lib.default_params(species="D2O", model="e3b3"))
    assert (p.imodel, p.ispecies) == (1, 3)


def test_engine_option_keys(lib, tmp_path):
    """The engine's own keys (no counterpart in the reference) parse from input.inp, default
    off, and refine_eigen (FP64 refinement steps) is range-checked."""
    from calcir_gb300 import CirError, finalize
    p = lib.default_params()
    assert (p.propagate_vectors, p.share_frames, p.refine_eigen) == (0, 0, 0)
    f = tmp_path / "input.inp"
    f.write_text("species H2O\nmodel tip4p2005\nrefine_eigen 2\nshare_frames 1\npropagate_vectors 1\n")
    p = finalize(lib.parse_input(str(f)))
    assert (p.propagate_vectors, p.share_frames, p.refine_eigen) == (1, 1, 2)
    for bad in (-1, 9):
        with pytest.raises(CirError, match="refine_eigen"):
            finalize(lib.default_params(species="H2O", refine_eigen=bad))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_sizes_match_reference_outputs(lib, case):
    meta, gold = load_golden(case)
    k = meta["keys"]
    p = lib.default_params(**k)
    ntcf, nom, nls = lib.result_sizes(p)
    assert ntcf == gold["irrtcf"].shape[0] and nom == gold["Pw"].shape[0] and nls == gold["irls"].shape[0]
    assert nom == O.nomega(golden_params(meta))


def test_frame_index_matches_oracle(lib):
    p = lib.default_params(nsamples=4, ntcfpoints=37, sampleEvery=0.37, beginTime=0.13, dt=0.02)
    table = lib.frame_table(p, 0.010)
    prm = {"sampleEvery": 0.37, "beginTime": 0.13, "dt": 0.02}
    want = [O.frame_index(prm, 0.010, s, k) for s in range(4) for k in range(37)]
    assert table.tolist() == want


def test_trajectory_round_trip(lib, tmp_path):
    xyz, box = lib.synth_trajectory(8, 5, seed=2)
    path = str(tmp_path / "t.cirtrj")
    lib.write_traj(path, xyz, box, 0.01)
    x2, b2, t2, fdt = lib.read_traj(path, 1, 3)
    assert np.array_equal(x2, xyz[1:4]) and np.allclose(b2, box) and np.float32(fdt) == np.float32(0.01)
    np.testing.assert_allclose(t2, np.float32(0.01) * np.arange(1, 4), rtol=1e-6)
    with pytest.raises(Exception):
        lib.read_traj(path, 4, 3)


# sha256 of the float32 positions of synth_trajectory(64, 150, seed=11): the generator uses
# only IEEE basic operations, so x86-64 and aarch64 produce the same bytes
SYNTH_SHA = "0bf4553671ecd027"


def test_synthetic_generator(lib):
    xyz, box = lib.synth_trajectory(64, 150, seed=11)
    assert hashlib.sha256(xyz.tobytes()).hexdigest()[:16] == SYNTH_SHA
    assert np.allclose(box, 1.2417)
    m = xyz.reshape(150, 64, 4, 3)
    oh1 = np.linalg.norm(m[:, :, 1] - m[:, :, 0], axis=-1)
    oh2 = np.linalg.norm(m[:, :, 2] - m[:, :, 0], axis=-1)
    om = np.linalg.norm(m[:, :, 3] - m[:, :, 0], axis=-1)
    assert np.allclose(oh1, 0.09572, atol=2e-6) and np.allclose(oh2, 0.09572, atol=2e-6)
    assert np.allclose(om, 0.01546, atol=2e-6)
    cosang = np.einsum("fmk,fmk->fm", m[:, :, 1] - m[:, :, 0], m[:, :, 2] - m[:, :, 0]) / oh1 / oh2
    assert np.allclose(np.degrees(np.arccos(cosang)), 104.52, atol=1e-3)
    # no O/H contact below 0.15 nm between molecules (minimum image)
    for f in (0, 75, 149):
        s = m[f, :, :3].reshape(-1, 3)
        d = s[:, None] - s[None]
        d -= 1.2417 * np.round(d / 1.2417)
        r = np.linalg.norm(d, axis=-1)
        same = np.repeat(np.arange(64), 3)
        r[same[:, None] == same[None]] = 9
        assert r.min() >= 0.15 - 1e-6
    # frames move: rms displacement per frame of order sigma_trans * sqrt(3)
    step = np.linalg.norm(m[1:, :, 0] - m[:-1, :, 0], axis=-1)
    step = np.minimum(step, 1.2417 - step)
    assert 0.002 < np.median(step) < 0.01
    xyz2, _ = lib.synth_trajectory(64, 3, seed=12)
    assert not np.array_equal(xyz2[0], xyz[0])


def test_write_outputs_formats(lib, tmp_path):
    """13 files with the reference's names and formats (calcIR.cu:843-919)."""
    meta, gold = load_golden("bend_hod_h2o")
    p = lib.default_params(**meta["keys"])
    p.outf = str(tmp_path / "ref").encode()
    ntcf, nom, nls = lib.result_sizes(p)
    res = {k: gold[f + "rtcf"][:, 1] + 1j * gold[f + "itcf"][:, 1] for k, f in
           (("tcf_ir", "ir"), ("tcf_vv", "vv"), ("tcf_vh", "vh"))}
    res.update(omega=gold["spdn"][:, 0], sw=gold["spdn"][:, 1], pw=gold["Pw"][:, 1], rw=gold["Rw"][:, 1],
               rmw=gold["Rmw"][:, 1], ls_omega=gold["irls"][:, 0], ls_ir=gold["irls"][:, 1],
               ls_vv=gold["vvls"][:, 1], ls_vh=gold["vhls"][:, 1])
    lib.write_outputs(p, res)
    names = sorted(os.listdir(tmp_path))
    assert names == sorted(f"ref_{s}.dat" for s in ["irrtcf", "iritcf", "vvrtcf", "vvitcf", "vhrtcf", "vhitcf",
                                                    "spdn", "Pw", "Rw", "Rmw", "irls", "vvls", "vhls"])
    head = open(tmp_path / "ref_irrtcf.dat").read()[:len(gold["irrtcf_text_head"])]
    assert head == bytes(gold["irrtcf_text_head"]).decode()
    for s in ["spdn", "Pw", "Rw", "Rmw", "irls"]:
        a = np.loadtxt(tmp_path / f"ref_{s}.dat")
        np.testing.assert_array_equal(np.nan_to_num(a, nan=-1), np.nan_to_num(gold[s], nan=-1))


def test_no_device_fails_loudly(lib):
    """Without a usable GPU the engine refuses to start: there is no CPU fallback."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from calcir_gb300 import CirError, Engine
    p = lib.default_params(species="H2O")
    with pytest.raises(CirError, match="NODEVICE|CUDA"):
        Engine(p, 256)
