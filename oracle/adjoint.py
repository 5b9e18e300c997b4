"""FP64 reference gradients of the spectrum-mismatch loss -- TEST INFRASTRUCTURE ONLY.

Only the tests may import this module.  The loss (the differentiation form's objective) is

    L(theta) = sum_rows (ls_ir - target_ir)^2 + sum_rows (ls_vv - target_vv)^2

over the printed lineshape rows (calcIR.cu:890-919) of a job computed with map and coupling
coefficients theta (13 values, THETA_NAMES, the coefficient arrays of calcIR.cu:1207-1242).
``fd_grad`` differentiates ``loss`` by central differences in FP64 (the reference gradient);
``adjoint_grad`` is the same adjoint the CUDA path implements, written in numpy:

  forward  psi_c(k) = U_k psi_c(k-1), psi_c(0) = m_c(0), U_k = V_k exp(i L_k dt/hbar) V_k^T;
           TCF(k) from m_b(k) . psi_a(k) (oracle.tcf_terms), lineshape by the C2R transform.
  backward g_k = dL/dTCF(k) (real and imaginary parts; the transpose of the C2R map), the
           adjoint lambda_c(k) = w_c(k) + U_{k+1} lambda_c(k+1) (U is complex symmetric),
           dL/dH_k = V_k Re(Phi_k o sum_c (V_k^T lambda_c(k)) (V_k^T psi_c(k-1))^T) V_k^T with
           Phi_mn the divided difference of exp(i x dt/hbar) at (lambda_m, lambda_n), written
           i tau exp(i tau (a+b)/2) sinc(tau (a-b)/2) so that equal eigenvalues are safe,
           then the chain rule through the maps to theta.
"""
from __future__ import annotations

import numpy as np

from . import oracle as O

THETA_NAMES = ["w0", "w1", "w2", "x0", "x1", "p0", "p1", "mup0", "mup1", "mup2", "wi0", "wi1", "wi2"]


def theta_of(mp: dict) -> np.ndarray:
    return np.array(list(mp["w"]) + list(mp["x"]) + list(mp["p"]) + list(mp["mup"]) + list(mp["wi"]), np.float64)


def maps_of(th) -> dict:
    th = [float(v) for v in th]
    return {"w": th[0:3], "x": th[3:5], "p": th[5:7], "mup": th[7:10], "wi": th[10:13]}


def _frame_quantities(xyz, box, prm, mp):
    E = O.field_projection(xyz, box, prm["natom_mol"], prm["nchrom_mol"], prm["imodel"])
    H, dip, pol = O.hamiltonian(xyz, box, E, prm["avef"], prm["natom_mol"], prm["nchrom_mol"], prm["ispecies"],
                                prm["map"], mp)
    return E, H, np.vstack([dip, pol])


def forward(prm, th, frames, boxes, fos, keep=False):
    """TCF sums (IR, VV) over origins, psi propagation; with keep, the per-step cache."""
    mp = maps_of(th)
    S, K = prm["nsamples"], prm["ntcfpoints"]
    tau = float(O.F32(prm["dt"])) / O.HBAR
    tir, tvv = np.zeros(K, complex), np.zeros(K, complex)
    cache = []
    for s in range(S):
        steps = []
        for k in range(K):
            f = fos[s * K + k]
            E, H, m = _frame_quantities(frames[f], boxes[f], prm, mp)
            lam, V = np.linalg.eigh(H)
            if k == 0:
                psi = m.astype(complex)
            else:
                psi = ((V * np.exp(1j * lam * tau)[None, :]) @ (V.T @ psi.T)).T
            ir, vv, _ = O.tcf_terms(psi, m)
            tir[k] += ir
            tvv[k] += vv
            if keep:
                steps.append({"f": f, "E": E, "lam": lam, "V": V, "m": m, "psi": psi})
        cache.append(steps)
    return tir, tvv, cache


def _rows(prm):
    """Indices of the printed lineshape rows in the C2R output, in file order."""
    ntcf, nz = prm["ntcfpoints"], prm["nzeros"]
    n = ntcf + nz
    dt = O.F32(prm["dt"])
    factor = O.F32(2 * O.PI * O.HBAR / float(dt * O.F32(n)))
    avef = O.F32(prm["avef"])
    idx = [i for i in range(n // 2, n) if O.F32(O.F32(-1 * (i - ntcf - nz)) * factor) + avef <= O.F32(prm["omegaStop"])]
    idx += [i for i in range(0, ntcf + nz // 2) if O.F32(O.F32(-1 * i) * factor) + avef >= O.F32(prm["omegaStart"])]
    return np.array(idx), float(factor * O.F32(n)), n


def damping(prm):
    S, K = prm["nsamples"], prm["ntcfpoints"]
    dt, t1 = float(O.F32(prm["dt"])), float(O.F32(prm["t1"]))
    return np.exp(-1.0 * np.arange(K) * dt / (2.0 * t1)) / (1.0 * S)


def lineshapes(prm, tir, tvv):
    """(IR, VV) lineshape rows from the TCF sums: damping, 1/nsamples, C2R, selection."""
    dcy = damping(prm)
    idx, norm, n = _rows(prm)
    return [O.c2r(t * dcy, n)[idx] / norm for t in (tir, tvv)]


def loss_of(prm, tir, tvv, targets):
    li, lv = lineshapes(prm, tir, tvv)
    return float(np.sum((li - targets[0]) ** 2) + np.sum((lv - targets[1]) ** 2))


def loss(prm, th, frames, boxes, fos, targets):
    tir, tvv, _ = forward(prm, th, frames, boxes, fos)
    return loss_of(prm, tir, tvv, targets)


def fd_grad(prm, th, frames, boxes, fos, targets, h=1e-5):
    """Central differences in FP64 with a relative step h (absolute h where theta is 0)."""
    th = np.asarray(th, np.float64)
    g = np.zeros_like(th)
    for p in range(len(th)):
        d = h * abs(th[p]) if th[p] != 0 else h
        tp, tm = th.copy(), th.copy()
        tp[p] += d
        tm[p] -= d
        g[p] = (loss(prm, tp, frames, boxes, fos, targets) - loss(prm, tm, frames, boxes, fos, targets)) / (2 * d)
    return g


def tcf_grad(prm, tir, tvv, targets):
    """dL/dTCF(k) for the IR and VV sums: complex g = dL/dRe + i dL/dIm."""
    K = prm["ntcfpoints"]
    dcy = damping(prm)
    idx, norm, n = _rows(prm)
    li, lv = lineshapes(prm, tir, tvv)
    out = []
    for ls, tg in ((li, targets[0]), (lv, targets[1])):
        dy = 2.0 * (ls - tg) / norm                      # dL/dy at the printed rows
        ang = 2 * np.pi * np.outer(idx, np.arange(K)) / n
        gr = (dy[:, None] * 2 * np.cos(ang)).sum(axis=0)
        gi = (dy[:, None] * -2 * np.sin(ang)).sum(axis=0)
        gr[0] = dy.sum()                                 # X_0 enters once, its imaginary part not at all
        gi[0] = 0.0
        out.append((gr + 1j * gi) * dcy)
    return out


def _map_derivatives(E, mp):
    """Per chromophore: values and d/dtheta (N, 13) of omega, x, p, mu'."""
    N = len(E)
    w = mp["w"][0] + mp["w"][1] * E + mp["w"][2] * E * E
    x = mp["x"][0] + mp["x"][1] * w
    p = mp["p"][0] + mp["p"][1] * w
    mup = mp["mup"][0] + mp["mup"][1] * E + mp["mup"][2] * E * E
    dw = np.zeros((N, 13)); dx = np.zeros((N, 13)); dp = np.zeros((N, 13)); dmup = np.zeros((N, 13))
    for q in range(3):
        dw[:, q] = E ** q
        dmup[:, 7 + q] = E ** q
    dx[:, :3] = mp["x"][1] * dw[:, :3]
    dx[:, 3] = 1.0
    dx[:, 4] = w
    dp[:, :3] = mp["p"][1] * dw[:, :3]
    dp[:, 5] = 1.0
    dp[:, 6] = w
    return w, x, p, mup, dw, dx, dp, dmup


def dtheta_H(G, xyz, box, E, prm, mp):
    """sum_ij G_ij dH_ij/dtheta for one frame."""
    box = np.asarray(box, np.float64)
    mol, n, Hpos, Opos, u = O.chromophores(xyz, box, prm["natom_mol"], prm["nchrom_mol"])
    w, x, p, mup, dw, dx, dp, dmup = _map_derivatives(E, mp)
    out = np.diag(G) @ dw
    if prm["ispecies"] in (1, 2):
        return out
    q = mup * x
    dq = dmup * x[:, None] + mup[:, None] * dx
    same = n[:, None] == n[None, :]
    np.fill_diagonal(same, False)
    t = O.min_image(Opos + 0.067 * u, box)
    dr = O.min_image(t[:, None, :] - t[None, :, :], box)
    r = np.linalg.norm(dr, axis=2)
    np.fill_diagonal(r, 1.0)
    nh = dr / r[:, :, None]
    R = r * O.BOHR_NM
    kap = (u @ u.T - 3.0 * np.einsum("ck,cdk->cd", u, nh) * np.einsum("dk,cdk->cd", u, nh)) / R ** 3 * O.CM_HARTREE
    inter = ~same
    np.fill_diagonal(inter, False)
    Gi = np.where(inter, G, 0.0)
    out += dq.T @ ((Gi + Gi.T) * kap) @ q
    # intramolecular pairs
    Gs = np.where(same, G, 0.0)
    wi = mp["wi"]
    coef = wi[0] + wi[1] * (E[:, None] + E[None, :])
    out[10] += np.sum(Gs * np.outer(x, x))
    out[11] += np.sum(Gs * (E[:, None] + E[None, :]) * np.outer(x, x))
    out[12] += np.sum(Gs * np.outer(p, p))
    out += dx.T @ (((Gs + Gs.T) * coef) @ x)
    out += dp.T @ (((Gs + Gs.T) * wi[2]) @ p)
    return out


def dtheta_m(gm, xyz, box, E, prm, mp):
    """sum_{b,i} gm[b, i] dm_b,i/dtheta for the nine vectors (dipole x, y, z; pol xx .. zx)."""
    mol, n, Hpos, Opos, u = O.chromophores(xyz, np.asarray(box, np.float64), prm["natom_mol"], prm["nchrom_mol"])
    w, x, p, mup, dw, dx, dp, dmup = _map_derivatives(E, mp)
    dq = dmup * x[:, None] + mup[:, None] * dx
    sq = gm[0] * u[:, 0] + gm[1] * u[:, 1] + gm[2] * u[:, 2]
    fac = np.stack([4.6 * u[:, 0] ** 2 + 1.0, 4.6 * u[:, 1] ** 2 + 1.0, 4.6 * u[:, 2] ** 2 + 1.0,
                    4.6 * u[:, 0] * u[:, 1], 4.6 * u[:, 1] * u[:, 2], 4.6 * u[:, 2] * u[:, 0]])
    sx = np.sum(gm[3:9] * fac, axis=0)
    return dq.T @ sq + dx.T @ sx


def _sources(g_ir, g_vv, m):
    """w_c = the coefficient vectors of psi_c in dL (9, N), from the TCF term structure."""
    w = np.zeros(m.shape, complex)
    w[0:3] = np.conj(g_ir) * m[0:3]
    s = m[3] + m[4] + m[5]
    for c in range(3, 6):
        w[c] = np.conj(g_vv) * (2 * m[c] + s) / 15.0
    w[6:9] = np.conj(g_vv) * 4 * m[6:9] / 15.0
    return w


def _m_grad(g_ir, g_vv, psi):
    """dL/dm_b(k) through the TCF terms at step k (9, N)."""
    gm = np.zeros(psi.shape)
    gm[0:3] = np.real(np.conj(g_ir) * psi[0:3])
    s = psi[3] + psi[4] + psi[5]
    for b in range(3, 6):
        gm[b] = np.real(np.conj(g_vv) * (2 * psi[b] + s) / 15.0)
    gm[6:9] = np.real(np.conj(g_vv) * 4 * psi[6:9] / 15.0)
    return gm


def _apply_U(st, vec, tau):
    V, lm = st["V"], st["lam"]
    return ((V * np.exp(1j * lm * tau)[None, :]) @ (V.T @ vec.T)).T


def adjoint_grad(prm, th, frames, boxes, fos, targets):
    """(L, dL/dtheta) by the adjoint, FP64."""
    mp = maps_of(th)
    tir, tvv, cache = forward(prm, th, frames, boxes, fos, keep=True)
    L = loss_of(prm, tir, tvv, targets)
    g_ir, g_vv = tcf_grad(prm, tir, tvv, targets)
    tau = float(O.F32(prm["dt"])) / O.HBAR
    K = prm["ntcfpoints"]
    grad = np.zeros(13)
    for steps in cache:
        lam_vec = None
        for k in range(K - 1, -1, -1):
            st = steps[k]
            w = _sources(g_ir[k], g_vv[k], st["m"])
            lam_vec = w if lam_vec is None else w + _apply_U(steps[k + 1], lam_vec, tau)
            gm = _m_grad(g_ir[k], g_vv[k], st["psi"])
            if k == 0:
                gm = gm + np.real(lam_vec)                   # psi_c(0) = m_c(0)
            f = st["f"]
            grad += dtheta_m(gm, frames[f], boxes[f], st["E"], prm, mp)
            if k >= 1:
                V, lm = st["V"], st["lam"]
                a = V.T @ lam_vec.T                          # (N, 9)
                b = V.T @ steps[k - 1]["psi"].T
                d = lm[:, None] - lm[None, :]
                phi = 1j * tau * np.exp(1j * tau * (lm[:, None] + lm[None, :]) / 2) * np.sinc(tau * d / (2 * np.pi))
                R = np.real(phi * (a @ b.T))
                G = V @ R @ V.T
                grad += dtheta_H(G, frames[f], boxes[f], st["E"], prm, mp)
    return L, grad
