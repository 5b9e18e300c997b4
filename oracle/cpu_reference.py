"""CPU timing port of the reference's per-frame loop -- TEST/BENCH INFRASTRUCTURE ONLY.

The reference (calcIR.cu) has no CPU implementation of its hot path: every frame it
builds H on the GPU, calls MAGMA ssyevd, builds a dense propagator and multiplies three
complex matrices, then evaluates 15 complex gemv + dot pairs (calcIR.cu:404-745).  This
module restates that per-frame work on the host with numpy/scipy's multithreaded
LAPACK/BLAS so bench.py can time the same algorithm on the GPU machine's host cores as the
reference-arm baseline:

  build      field projection (calcIR.cu:1020-1168) over the molecule pairs inside the
             cutoff (a periodic k-d tree finds them) and the Hamiltonian, dipoles and
             polarisabilities (calcIR.cu:1176-1406) as dense float32 arrays
  eigensolve LAPACK dsyevd in FP64 (scipy.linalg.eigh, driver "evd"), the divide-and-
             conquer driver the reference's magma_ssyevd_gpu mirrors (calcIR.cu:420-445)
  propagate  the dense propagator P, then cgemm x 3 (complex64) and the copy back into F
             (calcIR.cu:577-617)
  contract   15 cgemv + cdotu pairs (calcIR.cu:628-745)

Only bench.py's cpu_baseline leg and its --impl reference arm, and the tests, may call it.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import oracle as O

HBAR = 5.308837367
PAIRS = [(0, 0), (1, 1), (2, 2), (3, 3), (4, 4), (5, 5), (6, 6), (7, 7), (8, 8),
         (3, 4), (3, 5), (4, 3), (4, 5), (5, 3), (5, 4)]


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _inbox(x, L):
    y = np.mod(x, L)
    return np.where(y >= L, 0.0, y)


def field_projection(xyz, box, natom_mol=4, nchrom_mol=2, imodel=1):
    """E.u at every H (get_eproj_GPU, calcIR.cu:1020-1168) over the pairs inside the cutoff."""
    from scipy.spatial import cKDTree
    box = np.asarray(box, np.float64)
    mol, n, Hpos, Opos, u = O.chromophores(xyz, box, natom_mol, nchrom_mol)
    L = float(box[0])
    tree = cKDTree(_inbox(mol[:, 0], L), boxsize=L)
    hits = tree.query_ball_point(_inbox(Hpos, L), O.CUTOFF + 1e-5)
    c = np.repeat(np.arange(len(n)), [len(h) for h in hits])
    m = np.concatenate([np.asarray(h, np.int64) for h in hits]) if len(c) else np.zeros(0, np.int64)
    r = np.linalg.norm(O.min_image(mol[m, 0] - Hpos[c], box), axis=1)
    keep = (r <= O.CUTOFF) & (m != n[c])           # strict '>' skips (calcIR.cu:1106-1113)
    c, m = c[keep], m[keep]
    sites = [(mol[:, 1], 0.52), (mol[:, 2], 0.52)]
    if natom_mol >= 4:
        M = mol[:, 3]
        if imodel != 0:
            om = O.min_image(M - mol[:, 0], box)
            M = mol[:, 0] + 0.0150 * om / np.linalg.norm(om, axis=1)[:, None]
        sites.append((M, -1.04))
    E = np.zeros((len(n), 3))
    for s, q in sites:
        d = O.min_image(Hpos[c] - s[m], box) * O.BOHR_NM
        rr = np.linalg.norm(d, axis=1)
        np.add.at(E, c, (q / rr ** 3)[:, None] * d)
    return np.einsum("ck,ck->c", E, u)


def build(xyz, box, prm):
    """H (N, N) float32 and the nine dipole/polarisability rows (9, N) float32."""
    E = field_projection(xyz, box, prm["natom_mol"], prm["nchrom_mol"], prm["imodel"])
    box = np.asarray(box, np.float64)
    mp = O.maps(prm["map"], prm["ispecies"])
    mol, n, Hpos, Opos, u = O.chromophores(xyz, box, prm["natom_mol"], prm["nchrom_mol"])
    w = mp["w"][0] + mp["w"][1] * E + mp["w"][2] * E * E
    x = mp["x"][0] + mp["x"][1] * w
    p = mp["p"][0] + mp["p"][1] * w
    mup = mp["mup"][0] + mp["mup"][1] * E + mp["mup"][2] * E * E
    t = O.min_image(Opos + 0.067 * u, box).astype(np.float32)
    u32 = u.astype(np.float32)
    L = np.float32(box[0])
    N = len(E)
    H = np.zeros((N, N), np.float32)
    if prm["ispecies"] not in (1, 2):
        dr = t[:, None, :] - t[None, :, :]
        dr -= L * np.round(dr / L)
        r2 = np.einsum("cdk,cdk->cd", dr, dr)
        np.fill_diagonal(r2, 1.0)
        inv_r = 1.0 / np.sqrt(r2)
        un = np.einsum("ck,cdk->cd", u32, dr) * inv_r
        vn = np.einsum("dk,cdk->cd", u32, dr) * inv_r
        s = (x * mup).astype(np.float32)
        H = (u32 @ u32.T - 3.0 * un * vn) * (inv_r ** 3) * np.float32(1.0 / O.BOHR_NM ** 3 * O.CM_HARTREE)
        H *= np.outer(s, s)
        same = n[:, None] == n[None, :]
        intra = (mp["wi"][0] + mp["wi"][1] * (E[:, None] + E[None, :])) * np.outer(x, x) + mp["wi"][2] * np.outer(p, p)
        H[same] = intra[same]
    np.fill_diagonal(H, w - prm["avef"])
    dip = (u * (mup * x)[:, None]).T
    pol = np.stack([(4.6 * u[:, 0] ** 2 + 1.0) * x, (4.6 * u[:, 1] ** 2 + 1.0) * x,
                    (4.6 * u[:, 2] ** 2 + 1.0) * x, 4.6 * u[:, 0] * u[:, 1] * x,
                    4.6 * u[:, 1] * u[:, 2] * x, 4.6 * u[:, 2] * u[:, 0] * x])
    return H.astype(np.float32), np.vstack([dip, pol]).astype(np.float32)


def frame_step(xyz, box, prm, state):
    """One frame-step of the reference algorithm: build, dsyevd, dense propagator and three
    cgemm, 15 cgemv + cdotu."""
    import scipy.linalg as sl
    H, m = build(xyz, box, prm)                                     # calcIR.cu:404-406
    lam, V = sl.eigh(H.astype(np.float64), driver="evd", overwrite_a=True, check_finite=False)
    Vc = V.astype(np.complex64)
    mc = m.astype(np.complex64)
    if state.get("F") is None:                                     # k == 0: F = I
        state["F"] = np.eye(H.shape[0], dtype=np.complex64)
        state["m0"] = mc
    else:
        P = np.diag(np.exp(1j * lam * float(np.float32(prm["dt"])) / HBAR).astype(np.complex64))   # Pinit
        T = Vc @ P                                                 # cgemm 1
        P2 = T @ Vc.T                                              # cgemm 2
        state["F"] = P2 @ state["F"]                               # cgemm 3 + ccopy
    F, m0 = state["F"], state["m0"]
    return [np.dot(mc[b], F @ m0[a]) for a, b in PAIRS]             # 15 x (cgemv + cdotu)


def time_origin(frames, box, prm, frame_of_step, count: int) -> tuple[float, int]:
    """Seconds for the first `count` frame-steps of one time origin (frame_of_step[k] is the
    frame of step k) and the host thread count."""
    state = {}
    t = time.perf_counter()
    for k in range(count):
        frame_step(frames[frame_of_step[k]], box, prm, state)
    return time.perf_counter() - t, host_cores()
