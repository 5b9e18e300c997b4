"""GPU parity: every stage of the CUDA path against the FP64 oracle (or an FP64 numpy
statement of the same operation), the whole job against the oracle and the reference's
own golden outputs, and full-size (512 / 1024 molecules) properties.  All calls go
through the C ABI (libcalcir.so via ctypes)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN_CASES, golden_params, load_golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPEC_TOL = 1e-4    # relative L2 per spectrum, plain FP32 path vs FP64 oracle
HBAR = 5.308837367


def make_params(lib, prm, **extra):
    keys = {k: prm[k] for k in ("ntcfpoints", "nsamples", "sampleEvery", "omegaStep", "nchrom_mol", "nzeros",
                                "map", "dt", "t1", "avef", "beginTime", "omegaStart", "omegaStop")}
    model = "tip4p2005" if prm["imodel"] else "tip4p"
    species = ["H2O", "HOD/D2O", "HOD/H2O", "D2O"][prm["ispecies"]]
    keys.update(extra)
    return lib.default_params(model=model, species=species, **keys)


def near_cutoff(xyz, box, prm, eps=2e-5):
    """Chromophores with some O(m)..H(n) distance within eps of the field cutoff: FP32 and
    FP64 may disagree on including that molecule."""
    mol, n, Hpos, _, _ = O.chromophores(xyz, box, prm["natom_mol"], prm["nchrom_mol"])
    r = np.linalg.norm(O.min_image(mol[None, :, 0, :] - Hpos[:, None, :], np.asarray(box, float)), axis=2)
    return np.any(np.abs(r - O.CUTOFF) < eps, axis=1)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_build_hamiltonian(lib, case):
    meta, _ = load_golden(case)
    prm = golden_params(meta)
    xyz, box = lib.synth_trajectory(meta["nmol"], 4, seed=meta["seed"])
    with lib.Engine(make_params(lib, prm), xyz.shape[1]) as eng:
        H, E, dip, pol = eng.build_hamiltonian(xyz, box)
    for f in range(4):
        Eo, Ho, dipo, polo = O.frame(xyz[f], box, prm)
        ok = ~near_cutoff(xyz[f], box, prm)
        np.testing.assert_allclose(E[f][ok], Eo[ok], rtol=2e-5, atol=2e-7)
        sel = np.ix_(ok, ok)
        assert np.array_equal(H[f], H[f].T), "H must be exactly symmetric"
        np.testing.assert_allclose(H[f][sel], Ho[sel], rtol=1e-4, atol=2e-3)
        np.testing.assert_allclose(dip[f][:, ok], dipo[:, ok], rtol=1e-4, atol=1e-6)
        np.testing.assert_allclose(pol[f][:, ok], polo[:, ok], rtol=1e-4, atol=1e-6)


def _sym(rng, n, scale=1000.0):
    a = rng.standard_normal((n, n))
    return ((a + a.T) * (scale / np.sqrt(8 * n))).astype(np.float32)


def _check_eig(A, w, V, tol_scale=1.0):
    A64 = A.astype(np.float64)
    n = A.shape[0]
    nrm = max(np.abs(np.linalg.eigvalsh(A64)).max(), 1e-30)
    wref = np.linalg.eigvalsh(A64)
    assert np.all(np.diff(w) >= 0), "eigenvalues must ascend"
    assert np.abs(w - wref).max() <= 2e-6 * tol_scale * nrm * max(1.0, np.sqrt(n) / 4)
    V64 = V.astype(np.float64)
    assert np.abs(V64.T @ V64 - np.eye(n)).max() <= 2e-6 * tol_scale * max(1.0, np.sqrt(n))
    assert np.abs(A64 @ V64 - V64 * w[None, :]).max() <= 4e-6 * tol_scale * nrm * max(1.0, np.sqrt(n) / 4)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 64, 127, 128, 256, 257, 301, 432, 513, 686, 1023, 1024, 2048])
def test_eigh_random(lib, n):
    rng = np.random.default_rng(n)
    nmat = 3 if n <= 1024 else 1
    A = np.stack([_sym(rng, n) for _ in range(nmat)])
    with lib.Engine(lib.default_params(species="H2O"), 8) as eng:
        w, V = eng.eigh(A)
    for m in range(nmat):
        _check_eig(A[m], w[m], V[m])


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_eigh_rejects_non_finite_host_matrices(lib, bad):
    """A NaN or infinity in a host matrix is an error before any GPU work (the host check of
    cir_eigh); the context stays usable."""
    from calcir_gb300 import CirError
    rng = np.random.default_rng(3)
    A = np.stack([_sym(rng, 40) for _ in range(2)])
    A[1, 7, 3] = A[1, 3, 7] = bad
    with lib.Engine(lib.default_params(species="H2O"), 8) as eng:
        with pytest.raises(CirError, match="NaN or Inf"):
            eng.eigh(A)
        w, V = eng.eigh(A[:1])
    _check_eig(A[0], w[0], V[0])


@pytest.mark.parametrize("n", [96, 302])
def test_eigh_special_matrices(lib, n):
    """Zero, scaled identity, exact ties, a rank-one perturbation, diagonal, and a
    tridiagonal with exact zeros (96: unblocked tridiagonalisation; 302: blocked, with a
    padded leading dimension)."""
    rng = np.random.default_rng(5)
    cases = [np.zeros((n, n), np.float32), np.eye(n, dtype=np.float32) * 3.0,
             np.diag(np.repeat(np.arange(n // 8 + 1, dtype=np.float32), 8)[:n]),   # exact ties
             (np.eye(n) + np.outer(np.ones(n), np.ones(n)) / n).astype(np.float32),   # degenerate
             np.diag(rng.standard_normal(n).astype(np.float32)) * 500]
    t = np.zeros((n, n), np.float32)                                          # tridiagonal with zeros
    t[np.arange(n - 1), np.arange(1, n)] = t[np.arange(1, n), np.arange(n - 1)] = (np.arange(n - 1) % 5 != 0) * 7.0
    t += np.diag(np.linspace(-300, 300, n).astype(np.float32))
    cases.append(t)
    with lib.Engine(lib.default_params(species="H2O"), 8) as eng:
        w, V = eng.eigh(np.stack(cases))
    for m, A in enumerate(cases):
        _check_eig(A, w[m], V[m])


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
@pytest.mark.parametrize("n", [300, 1024])
def test_eigh_clustered_spectrum(lib, n, precision):
    """Eigenvalues in tight clusters (members 1e-4 apart, 1e-7 of the norm, up to 24 per
    cluster): every merge deflates long runs of consecutive close pairs by Givens rotations,
    which it applies to U as chains with one carried value per column.  The eigenpairs meet
    the bounds of the random matrices."""
    rng = np.random.default_rng(n + 11)
    lam = []
    while len(lam) < n:
        c = rng.uniform(-1000.0, 1000.0)
        lam.extend(c + 1e-4 * np.arange(min(int(rng.integers(1, 25)), n - len(lam))))
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    A = (Q * np.asarray(lam)) @ Q.T
    A = ((A + A.T) / 2).astype(np.float32)
    with lib.Engine(lib.default_params(species="H2O", precision=precision), 8) as eng:
        w, V = eng.eigh(A[None])
    _check_eig(A, w[0], V[0])


def test_propagate(lib):
    rng = np.random.default_rng(1)
    n, nprop, dt = 200, 3, 0.010
    A = np.stack([_sym(rng, n) for _ in range(nprop)])
    F = (rng.standard_normal((nprop, n, n)) + 1j * rng.standard_normal((nprop, n, n))).astype(np.complex64)
    with lib.Engine(lib.default_params(species="H2O"), 8) as eng:
        w, V = eng.eigh(A)
        out = eng.propagate(V, w, np.float32(dt), F)
    for m in range(nprop):
        V64 = V[m].astype(np.float64)
        ph = np.exp(1j * w[m].astype(np.float64) * np.float32(dt) / HBAR)
        ref = (V64 * ph[None, :]) @ (V64.T @ F[m].astype(np.complex128))
        assert O.rel_l2(out[m], ref) < 3e-6


def test_tcf_terms_and_spectral_density(lib):
    meta, _ = load_golden("small_h2o")
    prm = golden_params(meta)
    xyz, box = lib.synth_trajectory(meta["nmol"], 2, seed=meta["seed"])
    E0, H0, d0, p0 = O.frame(xyz[0], box, prm)
    E1, H1, d1, p1 = O.frame(xyz[1], box, prm)
    rng = np.random.default_rng(3)
    n = H0.shape[0]
    F = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) / np.sqrt(n)
    with lib.Engine(make_params(lib, prm), xyz.shape[1]) as eng:
        got = eng.tcf_terms(F.astype(np.complex64), d0.astype(np.float32), p0.astype(np.float32),
                            d1.astype(np.float32), p1.astype(np.float32))
        psi = (F.astype(np.complex64).astype(np.complex128) @ np.vstack([d0, p0]).astype(np.float32).T.astype(np.float64)).T
        ref = O.tcf_terms(psi, np.vstack([d1, p1]).astype(np.float32).astype(np.float64))
        for g, r in zip(got, ref):
            assert abs(g - r) <= 1e-5 * (abs(r) + 1e-3)
        lam, V = np.linalg.eigh(H0)
        Sw = eng.spectral_density(V.astype(np.float32), lam.astype(np.float32), d0.astype(np.float32))
    omega = prm["omegaStart"] + prm["omegaStep"] * np.arange(len(Sw))
    Mv = V.T @ d0.T
    g = HBAR / (np.float32(prm["t1"]) * 2.0)
    dw = omega[:, None] - (lam[None, :] + np.float32(prm["avef"]))
    ref = np.sum(np.sum(Mv * Mv, 1)[None, :] * g / (dw * dw + g * g) / O.PI, 1)
    assert O.rel_l2(Sw, ref) < 1e-5


@pytest.mark.parametrize("nzeros", [0, 1, 2, 97, 500, 25600])
def test_lineshape_fft(lib, nzeros):
    rng = np.random.default_rng(nzeros)
    ntcf = 150
    p = lib.default_params(species="H2O", ntcfpoints=ntcf, nzeros=nzeros, omegaStart=2000, omegaStop=5000,
                           avef=3415.0)
    tcf = (rng.standard_normal(ntcf) + 1j * rng.standard_normal(ntcf)) * np.exp(-np.arange(ntcf) / 40)
    prm = {"ntcfpoints": ntcf, "nzeros": nzeros, "dt": 0.010, "avef": 3415.0, "omegaStart": 2000,
           "omegaStop": 5000}
    with lib.Engine(p, 8) as eng:
        om, val = eng.lineshape(tcf)
    om_ref, val_ref = O.lineshape_rows(prm, O.c2r(tcf, ntcf + nzeros))
    np.testing.assert_array_equal(om, om_ref.astype(np.float32))
    assert O.rel_l2(val, val_ref) < 2e-6


def _frames_for(lib, meta):
    prm = golden_params(meta)
    xyz, box = lib.synth_trajectory(meta["nmol"], meta["nframes"], seed=meta["seed"])
    fos = np.array([O.frame_index(prm, meta["frame_dt"], s, k)
                    for s in range(prm["nsamples"]) for k in range(prm["ntcfpoints"])], np.int32)
    return prm, xyz, box, fos


def _compare_run(out, ref, prm, tol, name):
    for k in ("tcf_ir", "tcf_vv", "tcf_vh", "sw", "ls_ir", "ls_vv", "ls_vh"):
        e = O.rel_l2(out[k], ref[k])
        assert e < tol, (name, k, e)
    np.testing.assert_array_equal(out["omega"], np.asarray(ref["omega"], np.float32))
    np.testing.assert_array_equal(out["ls_omega"], np.asarray(ref["ls_omega"], np.float32))
    step = prm["omegaStep"]
    ntot = np.sum(ref["count"])
    assert abs(np.sum(out["pw"]) * step - 1) < 1e-5
    assert np.max(np.abs(np.cumsum(out["pw"]) - np.cumsum(ref["pw"]))) * step <= 4.0 / ntot + 1e-6
    for k in ("rw", "rmw"):
        a, b = np.nan_to_num(out[k] * out["pw"]), np.nan_to_num(ref[k] * ref["pw"])
        assert np.max(np.abs(np.cumsum(a) - np.cumsum(b))) <= 4.0 * np.abs(b).max() + 1e-6 * np.abs(b).sum()


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_run_matches_oracle_and_reference(lib, case):
    meta, gold = load_golden(case)
    prm, xyz, box, fos = _frames_for(lib, meta)
    with lib.Engine(make_params(lib, prm), xyz.shape[1]) as eng:
        out = eng.run(xyz, box, fos)
        st = eng.stats()
    assert st["kernel_launches"] > 0 and st["frame_steps"] == len(fos)
    assert out["bins_out_of_range"] == 0
    ref = O.run(prm, xyz, [box] * len(xyz), fos)
    _compare_run(out, ref, prm, SPEC_TOL, case)
    # and directly against the reference program's own outputs
    for k, f in (("tcf_ir", "ir"), ("tcf_vv", "vv"), ("tcf_vh", "vh")):
        g = gold[f + "rtcf"][:, 1] + 1j * gold[f + "itcf"][:, 1]
        assert O.rel_l2(out[k], g) < 2 * SPEC_TOL, (case, k)
    for k, f in (("ls_ir", "irls"), ("ls_vv", "vvls"), ("ls_vh", "vhls")):
        assert O.rel_l2(out[k], gold[f][:, 1]) < 2 * SPEC_TOL, (case, k)
        np.testing.assert_array_equal(O.as_printed(out["ls_omega"]), gold[f][:, 0])
    assert O.rel_l2(out["sw"], gold["spdn"][:, 1]) < 2 * SPEC_TOL


def test_run_full_propagation_matches_psi_oracle(lib):
    """The oracle's F-matrix and psi-vector propagations agree; the GPU path carries F."""
    meta, _ = load_golden("multi_d2o_map1")
    prm, xyz, box, fos = _frames_for(lib, meta)
    a = O.run(prm, xyz, [box] * len(xyz), fos, propagate="full")
    b = O.run(prm, xyz, [box] * len(xyz), fos, propagate="psi")
    for k in ("tcf_ir", "tcf_vv", "tcf_vh"):
        assert O.rel_l2(a[k], b[k]) < 1e-12


def test_dropin_executable(lib, tmp_path):
    """calcir input.inp writes the 13 files of the reference, matching its outputs."""
    meta, gold = load_golden("hod_d2o")
    xyz, box = lib.synth_trajectory(meta["nmol"], meta["nframes"], seed=meta["seed"])
    lib.write_traj(str(tmp_path / "traj.cirtrj"), xyz, box, 0.010)
    lines = ["xtcf traj.cirtrj", "outf ref", "natom_mol 4"] + [f"{k} {v}" for k, v in meta["keys"].items()]
    (tmp_path / "input.inp").write_text("\n".join(lines) + "\n")
    r = subprocess.run([lib.EXE_PATH, "input.inp"], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    for f in ["irrtcf", "iritcf", "vvrtcf", "vvitcf", "vhrtcf", "vhitcf", "spdn", "Pw", "Rw", "Rmw", "irls",
              "vvls", "vhls"]:
        a = np.loadtxt(tmp_path / f"ref_{f}.dat", ndmin=2)
        assert a.shape == gold[f].shape, f
        np.testing.assert_array_equal(a[:, 0], gold[f][:, 0])
        if f in ("Pw", "Rw", "Rmw"):
            continue
        assert O.rel_l2(a[:, 1], gold[f][:, 1]) < 2 * SPEC_TOL, f
    # the usage message and exit code of calcIR.cu:14-18
    r = subprocess.run([lib.EXE_PATH], stdout=subprocess.PIPE, text=True)
    assert r.returncode != 0 and "Usage" in r.stdout


def test_dropin_executable_reads_xtc(lib, tmp_path):
    """`xtcf traj.xtc` (a GROMACS trajectory, 1/1000 nm precision): the executable's spectra
    equal a run on the frames as decoded, and stay within the quantisation of the
    positions of the uncompressed run."""
    import ctypes as C
    meta, _ = load_golden("hod_d2o")
    xyz, box = lib.synth_trajectory(meta["nmol"], meta["nframes"], seed=meta["seed"])
    b = np.ascontiguousarray(np.broadcast_to(box, (xyz.shape[0], 3)), np.float32)
    t = (0.010 * np.arange(xyz.shape[0])).astype(np.float32)
    from calcir_gb300._lib import check, load
    check(load().cir_xtc_write(str(tmp_path / "traj.xtc").encode(), xyz.shape[1], xyz.shape[0],
                               C.c_void_p(xyz.ctypes.data), C.c_void_p(b.ctypes.data), C.c_void_p(t.ctypes.data),
                               C.c_float(1000.0)))
    lines = ["xtcf traj.xtc", "outf x", "natom_mol 4"] + [f"{k} {v}" for k, v in meta["keys"].items()]
    (tmp_path / "input.inp").write_text("\n".join(lines) + "\n")
    r = subprocess.run([lib.EXE_PATH, "input.inp"], cwd=tmp_path, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    dec = np.zeros_like(xyz)
    check(load().cir_traj_read(str(tmp_path / "traj.xtc").encode(), 0, xyz.shape[0], C.c_void_p(dec.ctypes.data),
                               None, None))
    assert np.abs(dec - xyz).max() <= 0.5e-3 + 1e-6
    prm, _, _, fos = _frames_for(lib, meta)
    with lib.Engine(make_params(lib, prm), xyz.shape[1]) as eng:
        out = eng.run(dec, box, fos)
    for f, k in (("irrtcf", "tcf_ir"), ("vvrtcf", "tcf_vv"), ("spdn", "sw")):
        a = np.loadtxt(tmp_path / f"x_{f}.dat", ndmin=2)[:, 1]
        ref = out[k].real if k.startswith("tcf") else out[k]
        assert O.rel_l2(a, ref) < 1e-5, f


@pytest.mark.parametrize("nmol", [512, 1024])
def test_full_size_eigen_and_unitarity(lib, nmol):
    """Full-size systems (1024 / 2048 chromophores): eigen-residuals, orthogonality, and
    F stays unitary over propagation steps (a size-independent property)."""
    nf = 6
    xyz, box = lib.synth_trajectory(nmol, nf, seed=21)
    p = lib.default_params(species="H2O", model="tip4p2005", avef=3415.0)
    with lib.Engine(p, xyz.shape[1]) as eng:
        H, E, dip, pol = eng.build_hamiltonian(xyz, box)
        w, V = eng.eigh(H)
        n = H.shape[-1]
        F = np.eye(n, dtype=np.complex64)
        for f in range(1, nf):
            F = eng.propagate(V[f], w[f], np.float32(0.010), F)
    for f in (0, nf - 1):
        _check_eig(H[f], w[f], V[f], tol_scale=2.0)
    F64 = F.astype(np.complex128)
    assert np.abs(F64.conj().T @ F64 - np.eye(n)).max() < 2e-4
    # reference identity at t = 0: IR tcf = sum_a |mu_a|^2 (calcIR.cu:628-647 with F = I)
    Eo, Ho, do, po = O.frame(xyz[0], box, {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0,
                                           "map": 0, "avef": 3415.0})
    np.testing.assert_allclose(np.sum(dip[0].astype(np.float64) ** 2), np.sum(do ** 2), rtol=1e-4)


_FULL_PRM = {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0, "map": 0, "ntcfpoints": 6,
             "nsamples": 2, "sampleEvery": 0.03, "dt": 0.010, "t1": 0.260, "avef": 3415.0, "omegaStart": 1000,
             "omegaStop": 5000, "omegaStep": 1, "nzeros": 2000, "beginTime": 0.0}
_FULL_REF = {}


def _full_case(lib, nmol):
    """nmol molecules, 2 origins x 6 steps, and the oracle's whole job on them (computed once)."""
    if nmol not in _FULL_REF:
        prm = _FULL_PRM
        xyz, box = lib.synth_trajectory(nmol, 10, seed=4)
        fos = np.array([O.frame_index(prm, 0.010, s, k) for s in range(2) for k in range(6)], np.int32)
        _FULL_REF[nmol] = (xyz, box, fos, O.run(prm, xyz, [box] * len(xyz), fos))
    return _FULL_REF[nmol]


@pytest.mark.parametrize("nmol", [512, 1024])
@pytest.mark.parametrize("precision", ["fp32", "bf16x3", "tf32"])
def test_run_full_size_against_oracle(lib, precision, nmol):
    """512 molecules (the full configuration's system, 1024 chromophores) and 1024 molecules
    (2048 chromophores, the largest order of the eigensolver), 2 origins x 6 steps, vs the
    oracle: the plain form within 1e-4 and the mixed forms (tensor-core propagation and
    eigenvector products) within 1e-3 per spectrum."""
    prm = _FULL_PRM
    xyz, box, fos, ref = _full_case(lib, nmol)
    with lib.Engine(make_params(lib, prm, precision=precision), xyz.shape[1]) as eng:
        out = eng.run(xyz, box, fos)
    errs = {k: O.rel_l2(out[k], ref[k]) for k in ("tcf_ir", "tcf_vv", "tcf_vh", "sw", "ls_ir", "ls_vv", "ls_vh")}
    print(f"{2 * nmol} chromophores {precision}:", {k: f"{v:.2e}" for k, v in errs.items()})
    _compare_run(out, ref, prm, SPEC_TOL if precision == "fp32" else MIXED_TOL, f"full{nmol}-" + precision)


def test_run_ten_origins_full_size(lib):
    """Ten time origins of 1024 chromophores (the headline's origin count), 3 steps each: the
    split-BF16 propagation runs each product as two whole waves of 128 x 256 tiles (nine
    origins) and the tenth origin in 128 x 64 tiles.  Against the FP32 form of the same run
    and the oracle; an error confined to the tail origin would still move the origin average
    by a tenth of its size."""
    prm = dict(_FULL_PRM, nsamples=10, ntcfpoints=3, sampleEvery=0.02)
    fos = np.array([O.frame_index(prm, 0.010, s, k) for s in range(10) for k in range(3)], np.int32)
    xyz, box = lib.synth_trajectory(512, int(fos.max()) + 1, seed=6)
    outs = {}
    for precision in ("fp32", "bf16x3"):
        with lib.Engine(make_params(lib, prm, precision=precision), xyz.shape[1]) as eng:
            outs[precision] = eng.run(xyz, box, fos)
    ref = O.run(prm, xyz, [box] * len(xyz), fos)
    for k in ("tcf_ir", "tcf_vv", "tcf_vh", "sw", "ls_ir", "ls_vv", "ls_vh"):
        em, ep = O.rel_l2(outs["bf16x3"][k], ref[k]), O.rel_l2(outs["fp32"][k], ref[k])
        print(f"ten origins {k}: bf16x3 {em:.2e}, fp32 {ep:.2e}")
        assert ep < SPEC_TOL and em < 2e-4, (k, em, ep)


@pytest.mark.parametrize("n", [200, 1024, 2048])
def test_propagate_tensor_core_tf32(lib, n):
    """The tcgen05 TF32 propagation against the FP64 statement of the same step; TF32
    inputs carry 11 significant bits, so the bound is 2e-3 relative."""
    rng = np.random.default_rng(n + 7)
    nprop, dt = 2, 0.010
    A = np.stack([_sym(rng, n) for _ in range(nprop)])
    F = (rng.standard_normal((nprop, n, n)) + 1j * rng.standard_normal((nprop, n, n))).astype(np.complex64)
    with lib.Engine(lib.default_params(species="H2O", precision="tf32"), 8) as eng:
        w, V = eng.eigh(A)
        out = eng.propagate(V, w, np.float32(dt), F)
    for m in range(nprop):
        V64 = V[m].astype(np.float64)
        ph = np.exp(1j * w[m].astype(np.float64) * np.float32(dt) / HBAR)
        ref = (V64 * ph[None, :]) @ (V64.T @ F[m].astype(np.complex128))
        err = O.rel_l2(out[m], ref)
        print(f"tf32 propagation step, n={n}: relative L2 error {err:.2e}")
        assert err < 2e-3, err
        assert err > 1e-7, "tensor-core path produced FP32-exact output: is it running?"


@pytest.mark.parametrize("n", [200, 1024, 2048])
def test_propagate_tensor_core_bf16x3(lib, n):
    """3-pass split-BF16 tcgen05 propagation: about 16 significant bits per operand."""
    rng = np.random.default_rng(n + 11)
    nprop, dt = 2, 0.010
    A = np.stack([_sym(rng, n) for _ in range(nprop)])
    F = (rng.standard_normal((nprop, n, n)) + 1j * rng.standard_normal((nprop, n, n))).astype(np.complex64)
    with lib.Engine(lib.default_params(species="H2O", precision="bf16x3"), 8) as eng:
        w, V = eng.eigh(A)
        out = eng.propagate(V, w, np.float32(dt), F)
    for m in range(nprop):
        V64 = V[m].astype(np.float64)
        ph = np.exp(1j * w[m].astype(np.float64) * np.float32(dt) / HBAR)
        ref = (V64 * ph[None, :]) @ (V64.T @ F[m].astype(np.complex128))
        err = O.rel_l2(out[m], ref)
        print(f"bf16x3 propagation step, n={n}: relative L2 error {err:.2e}")
        assert 1e-8 < err < 5e-5, err


MIXED_TOL = 1e-3   # relative L2 per spectrum for the mixed-precision forms


@pytest.mark.parametrize("precision", ["bf16x3", "tf32"])
@pytest.mark.parametrize("case", ["small_h2o", "multi_d2o_map1"])
def test_run_mixed_precision_forms(lib, case, precision):
    """The tensor-core forms against the FP64 oracle: every IR/Raman spectrum within
    1e-3 relative L2 (the bound the mixed-precision form is held to)."""
    meta, _ = load_golden(case)
    prm, xyz, box, fos = _frames_for(lib, meta)
    with lib.Engine(make_params(lib, prm, precision=precision), xyz.shape[1]) as eng:
        out = eng.run(xyz, box, fos)
    ref = O.run(prm, xyz, [box] * len(xyz), fos)
    errs = {k: O.rel_l2(out[k], ref[k]) for k in ("tcf_ir", "tcf_vv", "tcf_vh", "ls_ir", "ls_vv", "ls_vh", "sw")}
    print(case, precision, {k: f"{v:.2e}" for k, v in errs.items()})
    for k, v in errs.items():
        assert v < MIXED_TOL, (k, v)
