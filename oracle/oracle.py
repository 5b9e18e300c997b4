"""FP64 CPU oracle of calcIR's per-frame spectroscopy path -- TEST INFRASTRUCTURE ONLY.

This module restates, in double precision with numpy/LAPACK, the equations of the
reference program nicholashestand/calcIR (``calcIR.cu``).  Only the tests, the smoke
check of ``__graft_entry__`` and the CPU-baseline leg of ``bench.py`` may import it; the
product (``calcir_gb300``) never does.

Pinning: the parity of this restatement with the reference is checked against golden
outputs of the reference's own ``calcIR.cu``, compiled for the host from its unmodified
sources with shim headers for MAGMA, xdrfile and cuFFT (``oracle/build_ref.sh``), see
``tests/golden/make_golden.py`` and ``tests/test_oracle_golden.py``.

Coefficients that the reference stores in ``float`` variables (maps, cutoff, unit
conversions) are used with their float32 values; double literals (charges 0.52/1.04,
the 0.0150 nm M-site and 0.067 nm dipole offsets, the polarisability 4.6, hbar, pi) stay
double, as in the reference.
"""
from __future__ import annotations

import numpy as np

HBAR = 5.308837367          # calcIR.h:36
PI = 3.14159265359          # calcIR.h:37
F32 = np.float32
BOHR_NM = float(F32(18.8973))        # calcIR.cu:1036, 1197 (const float)
CM_HARTREE = float(F32(2.1947463e5))  # calcIR.cu:1198 (const float)
CUTOFF = float(F32(0.7831))           # calcIR.cu:1035 (const float)


def _f(x):
    return [float(F32(v)) for v in x]


def maps(imap: int, ispecies: int) -> dict:
    """Spectroscopic map coefficients, calcIR.cu:1207-1242."""
    h = ispecies in (0, 1)
    if imap == 0:
        w = [3670.2, -3541.7, -152677.0] if h else [2767.8, -2630.3, -102601.0]
        x = [0.19285, -1.7261e-5] if h else [0.16593, -2.0632e-5]
        p = [1.6466, 5.7692e-4] if h else [2.0475, 8.9108e-4]
        mup, wi = [0.1646, 11.39, 63.41], [-1361.0, 27165.0, -1.887]
    elif imap == 1:
        w = [3732.9, -3519.8, -153520.0] if h else [2748.2, -2572.2, -102980.0]
        x = [0.19318, -1.7248e-5] if h else [0.16598, -2.0752e-5]
        p = [1.6102, 5.8697e-4] if h else [1.9813, 9.1419e-4]
        mup, wi = [0.1622, 10.381, 137.6], [-1360.8, 27171.0, -1.887]
    else:
        raise ValueError("map must be 0 or 1")
    return {"w": _f(w), "x": _f(x), "p": _f(p), "mup": _f(mup), "wi": _f(wi)}


def round_half_away(x):
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def min_image(d, L):
    """minImage, calcIR.cu:1459-1463: dx - L*round(dx/L)."""
    return d - L * round_half_away(d / L)


def chromophores(xyz, box, natom_mol=4, nchrom_mol=2):
    """O and H of every chromophore and the OH unit vector (calcIR.cu:1046-1083, 1262-1286).

    The H of chromophore c is atom 1 + (c % 2) of molecule c // nchrom_mol."""
    xyz = np.asarray(xyz, np.float64)
    box = np.asarray(box, np.float64)
    nmol = xyz.shape[0] // natom_mol
    mol = xyz.reshape(nmol, natom_mol, 3)
    c = np.arange(nmol * nchrom_mol)
    n = c // nchrom_mol
    Hpos = mol[n, 1 + c % 2]
    Opos = mol[n, 0]
    u = min_image(Hpos - Opos, box)
    u /= np.linalg.norm(u, axis=1)[:, None]
    return mol, n, Hpos, Opos, u


def field_projection(xyz, box, natom_mol=4, nchrom_mol=2, imodel=1):
    """E.u at every H: get_eproj_GPU, calcIR.cu:1020-1168."""
    box = np.asarray(box, np.float64)
    mol, n, Hpos, Opos, u = chromophores(xyz, box, natom_mol, nchrom_mol)
    nmol = mol.shape[0]
    # cutoff on the O(m) .. H(n) distance, strict '>' skips (calcIR.cu:1106-1113)
    dOH = min_image(mol[None, :, 0, :] - Hpos[:, None, :], box)
    r = np.linalg.norm(dOH, axis=2)
    mask = (r <= CUTOFF) & (np.arange(nmol)[None, :] != n[:, None])
    sites = [(mol[:, 1], 0.52), (mol[:, 2], 0.52)]
    if natom_mol >= 4:
        M = mol[:, 3]
        if imodel != 0:   # M moved to 0.0150 nm along OM (calcIR.cu:1131-1146)
            om = min_image(M - mol[:, 0], box)
            M = mol[:, 0] + 0.0150 * om / np.linalg.norm(om, axis=1)[:, None]
        sites.append((M, -1.04))
    E = np.zeros((len(n), 3))
    for s, q in sites:
        d = min_image(Hpos[:, None, :] - s[None, :, :], box) * BOHR_NM
        rr = np.where(mask, np.linalg.norm(d, axis=2), 1.0)
        E += np.einsum("cm,cmk->ck", np.where(mask, q / rr ** 3, 0.0), d)
    return np.einsum("ck,ck->c", E, u)


def hamiltonian(xyz, box, eproj, avef, natom_mol=4, nchrom_mol=2, ispecies=0, imap=0, mp=None):
    """Exciton Hamiltonian, dipoles and polarisabilities: get_kappa_GPU, calcIR.cu:1176-1406.

    Returns H (N, N), dip (3, N) and pol (6, N) in the order xx, yy, zz, xy, yz, zx.
    ``mp`` overrides the map coefficients (a dict like ``maps`` returns)."""
    box = np.asarray(box, np.float64)
    mp = maps(imap, ispecies) if mp is None else mp
    mol, n, Hpos, Opos, u = chromophores(xyz, box, natom_mol, nchrom_mol)
    E = np.asarray(eproj, np.float64)
    w = mp["w"][0] + mp["w"][1] * E + mp["w"][2] * E * E          # calcIR.cu:1256
    x = mp["x"][0] + mp["x"][1] * w
    p = mp["p"][0] + mp["p"][1] * w
    mup = mp["mup"][0] + mp["mup"][1] * E + mp["mup"][2] * E * E
    t = min_image(Opos + 0.067 * u, box)                           # calcIR.cu:1288-1291
    N = len(E)
    H = np.zeros((N, N))
    if ispecies not in (1, 2):
        same = n[:, None] == n[None, :]
        intra = (mp["wi"][0] + mp["wi"][1] * (E[:, None] + E[None, :])) * np.outer(x, x) \
            + mp["wi"][2] * np.outer(p, p)                          # calcIR.cu:1339
        dr = min_image(t[:, None, :] - t[None, :, :], box)
        r = np.linalg.norm(dr, axis=2)
        np.fill_diagonal(r, 1.0)
        nh = dr / r[:, :, None]
        R = r * BOHR_NM
        uu = u @ u.T
        un = np.einsum("ck,cdk->cd", u, nh)
        vn = np.einsum("dk,cdk->cd", u, nh)
        tdc = (uu - 3.0 * un * vn) / R ** 3 * np.outer(x * mup, x * mup) * CM_HARTREE   # calcIR.cu:1397
        H = np.where(same, intra, tdc)
    np.fill_diagonal(H, w - avef)                                   # calcIR.cu:1327
    dip = (u * (mup * x)[:, None]).T                                # calcIR.cu:1294-1296
    pol = np.stack([(4.6 * u[:, 0] ** 2 + 1.0) * x, (4.6 * u[:, 1] ** 2 + 1.0) * x,
                    (4.6 * u[:, 2] ** 2 + 1.0) * x, 4.6 * u[:, 0] * u[:, 1] * x,
                    4.6 * u[:, 1] * u[:, 2] * x, 4.6 * u[:, 2] * u[:, 0] * x])   # calcIR.cu:1299-1304
    return H, dip, pol


def frame(xyz, box, prm: dict, mp=None):
    """Field, Hamiltonian, dipoles and polarisabilities of one frame."""
    E = field_projection(xyz, box, prm["natom_mol"], prm["nchrom_mol"], prm["imodel"])
    H, dip, pol = hamiltonian(xyz, box, E, prm["avef"], prm["natom_mol"], prm["nchrom_mol"],
                              prm["ispecies"], prm["map"], mp)
    return E, H, dip, pol


def tcf_terms(psi, mt):
    """IR, VV, VH increments from psi_a = F m_a(0) (9, N) and m_b(t) (9, N), calcIR.cu:628-745."""
    term = lambda a, b: np.dot(mt[b], psi[a])
    ir = term(0, 0) + term(1, 1) + term(2, 2)
    ii = term(3, 3) + term(4, 4) + term(5, 5)
    ij = term(6, 6) + term(7, 7) + term(8, 8)
    jj = term(3, 4) + term(3, 5) + term(4, 3) + term(4, 5) + term(5, 3) + term(5, 4)
    return ir, (3 * ii + jj + 4 * ij) / 15.0, (2 * ii - jj + 6 * ij) / 30.0


def nomega(prm):
    """calcIR.cu:94 -- float arithmetic truncated to int."""
    return int((F32(prm["omegaStop"]) - F32(prm["omegaStart"])) / F32(prm["omegaStep"]) + F32(1))


def c2r(X, n):
    """Unnormalised inverse real DFT with cuFFT's C2R convention (calcIR.cu:790-825)."""
    buf = np.zeros(n // 2 + 1, complex)
    m = min(len(X), n // 2 + 1)
    buf[:m] = X[:m]
    return np.fft.irfft(buf, n) * n


def lineshape_rows(prm, y):
    """Frequency axis and printed intensities of the lineshape files, calcIR.cu:890-919.

    The axis is evaluated in float32 exactly as the reference does."""
    ntcf, nz = prm["ntcfpoints"], prm["nzeros"]
    n = ntcf + nz
    dt = F32(prm["dt"])
    factor = F32(2 * PI * HBAR / float(dt * F32(n)))
    avef = F32(prm["avef"])
    om, val = [], []
    norm = float(factor * F32(n))
    for i in range(n // 2, n):
        freq = F32(F32(-1 * (i - ntcf - nz)) * factor) + avef
        if freq <= F32(prm["omegaStop"]):
            om.append(float(freq))
            val.append(y[i] / norm)
    for i in range(0, ntcf + nz // 2):
        freq = F32(F32(-1 * i) * factor) + avef
        if freq >= F32(prm["omegaStart"]):
            om.append(float(freq))
            val.append(y[i] / norm)
    return np.array(om), np.array(val)


def accumulate(prm: dict, frames, boxes, frame_of_step, samples=None, propagate="psi", keep_frames=False,
               mp=None):
    """The per-frame loop of the job (main, calcIR.cu:360-760) in FP64, over the time origins
    ``samples`` (default: all ``nsamples``): raw sums before the damping and normalisation.

    frames[f] is the (natoms, 3) position array of frame f, boxes[f] its box diagonal;
    frame_of_step[s*ntcf + k] selects the frame of step k of sample s.  propagate="full"
    carries the N x N matrix F like the reference; "psi" carries psi_a = F m_a(0) for the
    nine vectors, the same numbers at O(N^2) per step.  Sums of several calls over disjoint
    origin sets add up to the sums of one call over their union (``merge``)."""
    S, K = prm["nsamples"], prm["ntcfpoints"]
    samples = range(S) if samples is None else samples
    dt, t1, avef = float(F32(prm["dt"])), float(F32(prm["t1"])), float(F32(prm["avef"]))
    nom = nomega(prm)
    start, step = float(F32(prm["omegaStart"])), prm["omegaStep"]
    omega = np.array([float(F32(F32(prm["omegaStart"]) + F32(step * i))) for i in range(nom)])
    tcf = np.zeros((3, K), complex)
    Sw = np.zeros(nom)
    cnt = np.zeros(nom)
    ipr_acc = np.zeros(nom)
    mipr_acc = np.zeros(nom)
    oor = 0
    gamma = HBAR / (t1 * 2.0)
    ncm = prm["nchrom_mol"]
    per_frame = []
    N = None
    for s in samples:
        for k in range(K):
            f = frame_of_step[s * K + k]
            E, H, dip, pol = frame(frames[f], boxes[f], prm, mp)
            N = H.shape[0]
            lam, V = np.linalg.eigh(H)
            mvec = np.vstack([dip, pol])
            # frequency distribution (calcIR.cu:493-538)
            V2 = V * V
            ipr = 1.0 / np.sum(V2 * V2, axis=0)
            mipr = 1.0 / np.sum(V2.reshape(N // ncm, ncm, N).sum(axis=1) ** 2, axis=0)
            b = round_half_away((lam + avef - start) / step).astype(np.int64)
            ok = (b >= 0) & (b < nom)
            oor += int(np.count_nonzero(~ok))
            np.add.at(cnt, b[ok], 1.0)
            np.add.at(ipr_acc, b[ok], ipr[ok])
            np.add.at(mipr_acc, b[ok], mipr[ok])
            if k == 0:
                # spectral density (calcIR.cu:458-482, 1414-1444)
                Mv = V.T @ dip.T
                mu2 = np.sum(Mv * Mv, axis=1)
                dw = omega[:, None] - (lam[None, :] + avef)
                Sw += np.sum(mu2[None, :] * gamma / (dw * dw + gamma * gamma) / PI, axis=1)
                m0 = mvec.copy()
                if propagate == "full":
                    F = np.eye(N, dtype=complex)
                else:
                    psi = m0.astype(complex)
            else:
                ph = np.exp(1j * lam * dt / HBAR)
                if propagate == "full":
                    F = (V * ph[None, :]) @ (V.T @ F)          # calcIR.cu:596-617
                else:
                    psi = ((V * ph[None, :]) @ (V.T @ psi.T)).T
            if propagate == "full":
                psi_k = (F @ m0.T).T
            else:
                psi_k = psi
            ir, vv, vh = tcf_terms(psi_k, mvec)
            tcf[0, k] += ir
            tcf[1, k] += vv
            tcf[2, k] += vh
            if keep_frames:
                per_frame.append({"E": E, "H": H, "lam": lam, "dip": dip, "pol": pol})
    acc = {"tcf": tcf, "sw": Sw, "count": cnt, "ipr": ipr_acc, "mipr": mipr_acc, "oor": oor, "nchrom": N,
           "omega": omega}
    if keep_frames:
        acc["frames"] = per_frame
    return acc


def merge(parts):
    """Sum of the raw sums of ``accumulate`` calls over disjoint origin sets."""
    out = dict(parts[0])
    for p in parts[1:]:
        for k in ("tcf", "sw", "count", "ipr", "mipr", "oor"):
            out[k] = out[k] + p[k]
    return out


def finish(prm: dict, acc):
    """Damping, normalisation, the C2R transforms and the lineshape rows (calcIR.cu:777-839,
    890-919) of the raw sums over all ``nsamples`` origins."""
    S, K = prm["nsamples"], prm["ntcfpoints"]
    dt, t1 = float(F32(prm["dt"])), float(F32(prm["t1"]))
    step = prm["omegaStep"]
    N = acc["nchrom"]
    kk = np.arange(K)
    dcy = np.exp(-1.0 * kk * dt / (2.0 * t1)) / (1.0 * S)
    tcf = acc["tcf"] * dcy[None, :]
    n = K + prm["nzeros"]
    ls = [lineshape_rows(prm, c2r(tcf[q], n)) for q in range(3)]
    norm = N * S * K
    cnt = acc["count"]
    with np.errstate(invalid="ignore", divide="ignore"):
        pw = cnt / step / norm
        rw = (acc["ipr"] / step / norm) / pw
        rmw = (acc["mipr"] / step / norm) / pw
    out = {
        "tcf_ir": tcf[0], "tcf_vv": tcf[1], "tcf_vh": tcf[2],
        "omega": acc["omega"], "sw": acc["sw"] / S, "pw": pw, "rw": rw, "rmw": rmw,
        "ls_omega": ls[0][0], "ls_ir": ls[0][1], "ls_vv": ls[1][1], "ls_vh": ls[2][1],
        "bins_out_of_range": acc["oor"], "count": cnt,
    }
    if "frames" in acc:
        out["frames"] = acc["frames"]
    return out


def run(prm: dict, frames, boxes, frame_of_step, propagate="psi", keep_frames=False, mp=None):
    """The whole job (main, calcIR.cu:360-839) in FP64: ``accumulate`` over every time origin,
    then ``finish``."""
    return finish(prm, accumulate(prm, frames, boxes, frame_of_step, None, propagate, keep_frames, mp))


def frame_index(prm, frame_dt, s, k):
    """calcIR.cu:378-379 in float32: round((s*sampleEvery + beginTime + dt*k) / frame_dt)."""
    t = F32(F32(F32(s) * F32(prm["sampleEvery"])) + F32(prm["beginTime"])) + F32(F32(prm["dt"]) * F32(k))
    return int(round_half_away(F32(t / F32(frame_dt))))


def rel_l2(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def as_printed(x):
    """Values as the reference's "%g" output shows them (6 significant digits)."""
    return np.array([float("%g" % v) for v in np.asarray(x, np.float64)])
