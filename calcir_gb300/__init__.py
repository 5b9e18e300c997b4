"""GB300-native (sm_103a) implementation of calcIR's per-frame spectroscopy hot path.

The compute path is libcalcir.so (CUDA kernels behind the C ABI of include/calcir.h); the
drop-in executable is ``calcir_gb300/calcir input.inp``.  This module is a thin ctypes
host layer over that library for tests, benchmarks and Python users.  It has no CPU
implementation of the hot path: every call below runs CUDA kernels, and creating an
Engine fails when the library or a GPU is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from ._lib import (CIR_OK, EXE_PATH, LIB_PATH, PREC, CirError, Params, Result, Stats, Synth, TrajIn, check, load,
                   ptr)

__all__ = ["Engine", "CirError", "default_params", "parse_input", "synth_trajectory", "write_traj",
           "read_traj", "frame_table", "result_sizes", "write_outputs", "LIB_PATH", "EXE_PATH"]

_STR_KEYS = ("xtcf", "outf", "cptf", "model", "species")


def default_params(**kw) -> Params:
    """Reference defaults (calcIR.cu:36-59) updated with ``kw`` (input.inp key names)."""
    p = Params()
    check(load().cir_params_default(C.byref(p)))
    for k, v in kw.items():
        if k in _STR_KEYS:
            setattr(p, k, v.encode() if isinstance(v, str) else v)
        elif k == "precision" and isinstance(v, str):
            p.precision = PREC[v]
        else:
            setattr(p, k, v)
    return p


def parse_input(path: str, base: Params | None = None) -> Params:
    """Parse an input.inp file with the reference's key semantics (calcIR.cu:1539-1643)."""
    p = base if base is not None else default_params()
    check(load().cir_params_parse_file(path.encode(), C.byref(p)))
    return p


def finalize(p: Params) -> Params:
    check(load().cir_params_finalize(C.byref(p)))
    return p


def result_sizes(p: Params) -> tuple[int, int, int]:
    a, b, c = C.c_int(), C.c_int(), C.c_int()
    check(load().cir_result_sizes(C.byref(p), C.byref(a), C.byref(b), C.byref(c)))
    return a.value, b.value, c.value


def frame_table(p: Params, frame_dt: float) -> np.ndarray:
    """Frame index of every (sample, step), calcIR.cu:378-379."""
    out = np.empty(p.nsamples * p.ntcfpoints, np.int32)
    f = C.c_int()
    lib = load()
    for s in range(p.nsamples):
        for k in range(p.ntcfpoints):
            check(lib.cir_frame_index(C.byref(p), C.c_float(frame_dt), s, k, C.byref(f)))
            out[s * p.ntcfpoints + k] = f.value
    return out


def synth_trajectory(nmol: int, nframes: int, seed: int = 1, **kw) -> tuple[np.ndarray, np.ndarray]:
    """Seeded synthetic water box: positions (nframes, 4*nmol, 3) float32 and box (3,)."""
    s = Synth()
    check(load().cir_synth_default(C.byref(s), nmol))
    s.seed = seed
    for k, v in kw.items():
        setattr(s, k, v)
    xyz = np.empty((nframes, 4 * nmol, 3), np.float32)
    box = np.empty(3, np.float32)
    rej = C.c_longlong()
    check(load().cir_synth_trajectory(C.byref(s), nframes, ptr(xyz), ptr(box), C.byref(rej)))
    return xyz, box


def write_traj(path: str, xyz: np.ndarray, boxes: np.ndarray, frame_dt: float, times=None) -> None:
    xyz = np.ascontiguousarray(xyz, np.float32)
    boxes = np.ascontiguousarray(np.broadcast_to(boxes, (xyz.shape[0], 3)), np.float32)
    t = None if times is None else np.ascontiguousarray(times, np.float32)
    check(load().cir_traj_write(path.encode(), xyz.shape[1], xyz.shape[0], C.c_float(frame_dt), ptr(t),
                                ptr(boxes), ptr(xyz)))


def read_traj(path: str, first: int = 0, count: int | None = None):
    natoms, nframes, fdt = C.c_int(), C.c_int(), C.c_float()
    check(load().cir_traj_info(path.encode(), C.byref(natoms), C.byref(nframes), C.byref(fdt)))
    count = nframes.value - first if count is None else count
    xyz = np.empty((count, natoms.value, 3), np.float32)
    boxes = np.empty((count, 3), np.float32)
    times = np.empty(count, np.float32)
    check(load().cir_traj_read(path.encode(), first, count, ptr(xyz), ptr(boxes), ptr(times)))
    return xyz, boxes, times, fdt.value


def write_outputs(p: Params, res: dict) -> None:
    """Write the 13 output files of a result dictionary (calcIR.cu:843-919)."""
    keep = []

    def dp(a, dt):
        a = np.ascontiguousarray(a, dt)
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(C.c_double if dt == np.float64 else C.c_float))

    r = Result()
    for k in ("tcf_ir", "tcf_vv", "tcf_vh"):
        setattr(r, k, dp(np.stack([res[k].real, res[k].imag], 1).ravel(), np.float64))
    for k in ("omega", "sw", "pw", "rw", "rmw", "ls_omega", "ls_ir", "ls_vv", "ls_vh"):
        setattr(r, k, dp(res[k], np.float32))
    r.nls = len(res["ls_omega"])
    check(load().cir_write_outputs(C.byref(p), C.byref(r)))


def _result_dict(bufs: dict, r) -> dict:
    out = {k: (bufs[k][0::2] + 1j * bufs[k][1::2]) if k.startswith("tcf") else bufs[k] for k in bufs}
    for k in ("ls_omega", "ls_ir", "ls_vv", "ls_vh"):
        out[k] = out[k][:r.nls]
    out["bins_out_of_range"] = r.bins_out_of_range
    out["frame_steps_per_s"] = r.frame_steps_per_s
    return out


class Engine:
    """One GPU context (cir_ctx) for a system of ``natoms`` atoms."""

    def __init__(self, params: Params, natoms: int):
        self.lib = load()
        self.p = params
        h = C.c_void_p()
        check(self.lib.cir_create(C.byref(params), natoms, C.byref(h)))
        self.h = h
        q = Params.from_buffer_copy(params)
        check(self.lib.cir_params_finalize(C.byref(q)))
        self.natoms = natoms
        self.nmol = natoms // q.natom_mol
        self.n = self.nmol * q.nchrom_mol
        self.params = q

    def close(self):
        if getattr(self, "h", None):
            self.lib.cir_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_handle: int | None):
        check(self.lib.cir_set_stream(self.h, C.c_void_p(stream_handle) if stream_handle else None))

    def synchronize(self):
        check(self.lib.cir_synchronize(self.h))

    def stats(self) -> dict:
        s = Stats()
        check(self.lib.cir_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def reset_stats(self):
        check(self.lib.cir_reset_stats(self.h))

    def build_hamiltonian(self, xyz, box):
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, self.natoms, 3)
        nf = xyz.shape[0]
        box = np.ascontiguousarray(np.broadcast_to(np.asarray(box, np.float32), (nf, 3)))
        n = self.n
        H = np.empty((nf, n, n), np.float32)
        E = np.empty((nf, n), np.float32)
        dip = np.empty((nf, 3, n), np.float32)
        pol = np.empty((nf, 6, n), np.float32)
        check(self.lib.cir_build_hamiltonian(self.h, nf, ptr(xyz), ptr(box), ptr(H), ptr(E), ptr(dip), ptr(pol)))
        return H, E, dip, pol

    def eigh(self, A):
        """Eigenvalues (ascending) and eigenvectors (columns) of a batch of symmetric matrices."""
        A = np.array(A, np.float32, copy=True)
        single = A.ndim == 2
        A = A.reshape(-1, A.shape[-1], A.shape[-1])
        n = A.shape[-1]
        w = np.empty((A.shape[0], n), np.float32)
        # the library returns column j in A[m][j][:]
        check(self.lib.cir_eigh(self.h, A.shape[0], n, ptr(A), ptr(w)))
        V = np.ascontiguousarray(np.swapaxes(A, 1, 2))
        return (w[0], V[0]) if single else (w, V)

    def tridiag_sbr(self, A):
        """Two-stage reduction to tridiagonal form: (d, e, ms) with d, e [nmat][n] and the
        device times of the two stages (dense -> band, band -> tridiagonal) in ms."""
        A = np.ascontiguousarray(A, np.float32)
        A = A.reshape(-1, A.shape[-1], A.shape[-1])
        n = A.shape[-1]
        d = np.empty((A.shape[0], n), np.float32)
        e = np.empty((A.shape[0], n), np.float32)
        ms = np.zeros(2, np.float32)
        check(self.lib.cir_tridiag_sbr(self.h, A.shape[0], n, ptr(A), ptr(d), ptr(e), ptr(ms)))
        return d, e, ms

    def propagate(self, V, w, dt, F):
        """F <- V diag(exp(i w dt/hbar)) V^T F; V holds eigenvectors as columns."""
        V = np.asarray(V, np.float32)
        single = V.ndim == 2
        V = V.reshape(-1, V.shape[-1], V.shape[-1])
        n = V.shape[-1]
        Vc = np.ascontiguousarray(np.swapaxes(V, 1, 2))        # column j contiguous
        w = np.ascontiguousarray(np.asarray(w, np.float32).reshape(-1, n))
        Fi = np.array(F, np.complex64, copy=True, order="C").reshape(-1, n, n)   # updated in place by the library
        Fr = Fi.view(np.float32)
        check(self.lib.cir_propagate(self.h, V.shape[0], n, ptr(Vc), ptr(w), C.c_float(dt), ptr(Fr)))
        out = Fr.view(np.complex64)
        return out[0] if single else out

    def tcf_terms(self, F, dip0, pol0, dip, pol):
        n = F.shape[-1]
        Fr = np.ascontiguousarray(np.asarray(F, np.complex64)).view(np.float32)
        out = np.zeros(6, np.float64)
        arrs = [np.ascontiguousarray(a, np.float32) for a in (dip0, pol0, dip, pol)]
        check(self.lib.cir_tcf_terms(self.h, n, ptr(Fr), *[ptr(a) for a in arrs], ptr(out)))
        return out[0] + 1j * out[1], out[2] + 1j * out[3], out[4] + 1j * out[5]

    def spectral_density(self, V, w, dip):
        n = V.shape[-1]
        nom = result_sizes(self.params)[1]
        Sw = np.zeros(nom, np.float32)
        Vc = np.ascontiguousarray(np.asarray(V, np.float32).T)
        w32 = np.ascontiguousarray(w, np.float32)
        d32 = np.ascontiguousarray(dip, np.float32)
        check(self.lib.cir_spectral_density(self.h, n, ptr(Vc), ptr(w32), ptr(d32), ptr(Sw)))
        return Sw

    def lineshape(self, tcf_damped):
        t = np.ascontiguousarray(np.stack([np.real(tcf_damped), np.imag(tcf_damped)], 1), np.float64)
        nls = result_sizes(self.params)[2]
        om = np.empty(nls, np.float32)
        val = np.empty(nls, np.float32)
        cnt = C.c_int()
        check(self.lib.cir_lineshape(self.h, ptr(t), ptr(om), ptr(val), C.byref(cnt)))
        return om[:cnt.value], val[:cnt.value]

    def run(self, xyz, boxes, frame_of_step=None, nframes: int | None = None) -> dict:
        """The whole job (cir_run): xyz (nframes, natoms, 3), boxes (nframes, 3) or (3,).

        xyz and boxes may also be device (or pinned host) addresses given as ints, with
        ``nframes`` stating how many frames they hold."""
        if isinstance(xyz, int):
            nf = int(nframes)
        else:
            xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, self.natoms, 3)
            nf = xyz.shape[0]
        if not isinstance(boxes, int):
            boxes = np.ascontiguousarray(np.broadcast_to(np.asarray(boxes, np.float32), (nf, 3)))
        fos = None if frame_of_step is None else np.ascontiguousarray(frame_of_step, np.int32)
        ntcf, nom, nls = result_sizes(self.params)
        bufs = {k: np.zeros(2 * ntcf, np.float64) for k in ("tcf_ir", "tcf_vv", "tcf_vh")}
        bufs.update({k: np.zeros(nom, np.float32) for k in ("omega", "sw", "pw", "rw", "rmw")})
        bufs.update({k: np.zeros(nls, np.float32) for k in ("ls_omega", "ls_ir", "ls_vv", "ls_vh")})
        r = Result()
        for k, a in bufs.items():
            setattr(r, k, a.ctypes.data_as(C.POINTER(C.c_double if a.dtype == np.float64 else C.c_float)))
        check(self.lib.cir_run(self.h, nf, ptr(xyz), ptr(boxes), ptr(fos), C.byref(r)))
        return _result_dict(bufs, r)

    def get_coeffs(self) -> np.ndarray:
        """The 13 map and coupling coefficients (w0 w1 w2 x0 x1 p0 p1 mup0 mup1 mup2 wi0 wi1 wi2)."""
        t = np.zeros(13, np.float32)
        check(self.lib.cir_get_coeffs(self.h, ptr(t)))
        return t

    def set_coeffs(self, theta) -> None:
        t = np.ascontiguousarray(theta, np.float32)
        check(self.lib.cir_set_coeffs(self.h, ptr(t)))

    def loss_grad(self, xyz, boxes, frame_of_step, target_ir, target_vv) -> tuple[float, np.ndarray]:
        """(L, dL/dtheta) of L = sum (ls_ir - target_ir)^2 + (ls_vv - target_vv)^2 over the printed
        lineshape rows (cir_loss_grad, the adjoint through propagation and eigendecomposition)."""
        xyz = np.ascontiguousarray(xyz, np.float32).reshape(-1, self.natoms, 3)
        nf = xyz.shape[0]
        boxes = np.ascontiguousarray(np.broadcast_to(np.asarray(boxes, np.float32), (nf, 3)))
        fos = None if frame_of_step is None else np.ascontiguousarray(frame_of_step, np.int32)
        ti = np.ascontiguousarray(target_ir, np.float32)
        tv = np.ascontiguousarray(target_vv, np.float32)
        loss = C.c_double()
        grad = np.zeros(13, np.float64)
        check(self.lib.cir_loss_grad(self.h, nf, ptr(xyz), ptr(boxes), ptr(fos), ptr(ti), ptr(tv), len(ti),
                                     C.byref(loss), ptr(grad)))
        return loss.value, grad

    def run_multi(self, trajectories) -> list[dict]:
        """Many trajectories, boxes of uneven size allowed (cir_run_multi): ``trajectories``
        is a list of (xyz (nframes, natoms, 3), boxes (nframes, 3) or (3,), frame_of_step or
        None); xyz and boxes may be numpy arrays or contiguous float32 device tensors (boxes
        then (nframes, 3)).  Returns one result dict per trajectory, as ``run`` would."""
        keep, tin = [], (TrajIn * len(trajectories))()
        for i, (xyz, boxes, fos) in enumerate(trajectories):
            if hasattr(xyz, "data_ptr"):     # device tensors (contiguous float32), used in place
                nf, na = int(xyz.shape[0]), int(xyz.shape[1])
                px, pb = xyz.data_ptr(), boxes.data_ptr()
            else:
                xyz = np.ascontiguousarray(xyz, np.float32)
                nf, na = xyz.shape[0], xyz.shape[1]
                boxes = np.ascontiguousarray(np.broadcast_to(np.asarray(boxes, np.float32), (nf, 3)))
                px, pb = xyz, boxes
            fos = None if fos is None else np.ascontiguousarray(fos, np.int32)
            keep += [xyz, boxes, fos]
            tin[i].natoms, tin[i].nframes = na, nf
            tin[i].xyz, tin[i].box, tin[i].frame_of_step = ptr(px), ptr(pb), ptr(fos)
        ntcf, nom, nls = result_sizes(self.params)
        allbufs, rs = [], (Result * len(trajectories))()
        for i in range(len(trajectories)):
            bufs = {k: np.zeros(2 * ntcf, np.float64) for k in ("tcf_ir", "tcf_vv", "tcf_vh")}
            bufs.update({k: np.zeros(nom, np.float32) for k in ("omega", "sw", "pw", "rw", "rmw")})
            bufs.update({k: np.zeros(nls, np.float32) for k in ("ls_omega", "ls_ir", "ls_vv", "ls_vh")})
            for k, a in bufs.items():
                setattr(rs[i], k, a.ctypes.data_as(C.POINTER(C.c_double if a.dtype == np.float64 else C.c_float)))
            allbufs.append(bufs)
        check(self.lib.cir_run_multi(self.h, len(trajectories), tin, rs))
        return [_result_dict(allbufs[i], rs[i]) for i in range(len(trajectories))]
