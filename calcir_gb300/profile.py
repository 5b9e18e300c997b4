"""Small drivers for profiling single stages of the CUDA path (run under ncu or with
CIR_EIGH_PROFILE=1 for the eigensolver's per-phase timers).

    python -m calcir_gb300.profile eigh --nmol 512 --batch 152
    python -m calcir_gb300.profile prop --n 1024 --nprop 10
    python -m calcir_gb300.profile run --nmol 512 --nsamples 10 --ntcf 250
    python -m calcir_gb300.profile run --nmol 512 --nsamples 10 --ntcf 50 --propagate-vectors 1
    python -m calcir_gb300.profile grad --nmol 256 --nsamples 2 --ntcf 32
    python -m calcir_gb300.profile noalloc --nmol 256 --batch 16
    python -m calcir_gb300.profile sbr --nmol 512 --batch 2500
    python -m calcir_gb300.profile multi --sizes 128,216,343,512 --ntraj 4 --ntcf 200

Every stage goes through the C ABI (libcalcir.so)."""
from __future__ import annotations

import argparse
import time

import numpy as np

import calcir_gb300 as cg


def eigh(nmol: int, batches: list[int], seed: int = 3) -> None:
    xyz, box = cg.synth_trajectory(nmol, 8, seed=seed)
    p = cg.default_params(model="tip4p2005", species="H2O", avef=3415.0)
    with cg.Engine(p, xyz.shape[1]) as eng:
        H, _, _, _ = eng.build_hamiltonian(xyz, box)
        for nb in batches:
            A = np.ascontiguousarray(np.broadcast_to(H[np.arange(nb) % 8], (nb,) + H.shape[1:]))
            t = time.time()
            eng.eigh(A)
            dt = time.time() - t
            print(f"eigh N={H.shape[-1]} batch {nb}: {dt:.3f} s wall ({nb / dt:.1f} matrices/s incl. copies)", flush=True)


def prop(n: int, nprop: int, precision: str = "fp32") -> None:
    rng = np.random.default_rng(0)
    a = rng.standard_normal((n, n)).astype(np.float32)
    A = (a + a.T) * np.float32(300 / np.sqrt(8 * n))
    with cg.Engine(cg.default_params(species="H2O", precision=precision), 8) as eng:
        w, V = eng.eigh(A)
        F = np.broadcast_to(np.eye(n, dtype=np.complex64), (nprop, n, n))
        out = eng.propagate(np.broadcast_to(V, (nprop, n, n)), np.broadcast_to(w, (nprop, n)), 0.01, F)
    print(f"prop N={n} x {nprop}: max |F| {np.abs(out).max():.4f}", flush=True)


def run(nmol: int, nsamples: int, ntcf: int, precision: str = "fp32", **options) -> None:
    """One job; autotune=0 keeps the autotuner's trial launches out of a capture."""
    p = cg.default_params(model="tip4p2005", species="H2O", ntcfpoints=ntcf, nsamples=nsamples, sampleEvery=2.0,
                          avef=3415.0, omegaStart=1000, omegaStop=5000, omegaStep=1, precision=precision, **options)
    fos = cg.frame_table(p, 0.010)
    xyz, box = cg.synth_trajectory(nmol, int(fos.max()) + 1, seed=1)
    with cg.Engine(p, xyz.shape[1]) as eng:
        out = eng.run(xyz, box, fos)
        print(f"run nmol {nmol}: {out['frame_steps_per_s']:.1f} frame-steps/s", eng.stats(), flush=True)


def multi(sizes: list[int], ntraj: int, ntcf: int) -> None:
    """One cir_run_multi job in the split-BF16 form over boxes of the given sizes (ntraj
    trajectories each, one origin of ntcf points), the autotuner off: the joint
    tridiagonalisation and propagation launches."""
    trajs = []
    for nmol in sizes:
        for t in range(ntraj):
            xyz, box = cg.synth_trajectory(nmol, ntcf, seed=1000 + 7 * nmol + t)
            trajs.append((xyz, box, None))
    p = cg.default_params(model="tip4p2005", species="H2O", ntcfpoints=ntcf, nsamples=1, sampleEvery=2.0,
                          avef=3415.0, omegaStart=2000, omegaStop=5000, omegaStep=1, precision="bf16x3", autotune=0)
    with cg.Engine(p, 4 * sizes[0]) as eng:
        eng.run_multi(trajs)
        print(f"multi {sizes} x {ntraj}:", eng.stats(), flush=True)


def sbr(nmol: int, nb: int, reps: int = 3) -> None:
    """The two-stage reduction to tridiagonal form (cir_tridiag_sbr) on nb water Hamiltonians
    (8 distinct frames repeated): the device times of its two stages."""
    xyz, box = cg.synth_trajectory(nmol, 8, seed=3)
    p = cg.default_params(model="tip4p2005", species="H2O", avef=3415.0)
    with cg.Engine(p, xyz.shape[1]) as eng:
        H, _, _, _ = eng.build_hamiltonian(xyz, box)
        A = np.ascontiguousarray(np.broadcast_to(H[np.arange(nb) % 8], (nb,) + H.shape[1:]))
        for r in range(reps):
            d, e, ms = eng.tridiag_sbr(A)
            print(f"sbr N={H.shape[-1]} batch {nb}: dense -> band {ms[0]:.1f} ms, band -> tridiagonal {ms[1]:.1f} ms",
                  flush=True)


def noalloc(nmol: int, nb: int) -> None:
    """cir_eigh_noalloc on device copies of water Hamiltonians (the implicit-QR eigensolver
    path: k_eigh_tq, k_eigh_formq, k_eigh_qr)."""
    import ctypes as C
    import torch
    from calcir_gb300._lib import check, load
    xyz, box = cg.synth_trajectory(nmol, 8, seed=3)
    p = cg.default_params(model="tip4p2005", species="H2O", avef=3415.0)
    with cg.Engine(p, xyz.shape[1]) as eng:
        H, _, _, _ = eng.build_hamiltonian(xyz, box)
    n = H.shape[-1]
    A = torch.from_numpy(np.ascontiguousarray(H[np.arange(nb) % 8])).cuda()
    w = torch.empty((nb, n), dtype=torch.float32, device="cuda")
    check(load().cir_eigh_noalloc(nb, n, C.c_void_p(A.data_ptr()), C.c_void_p(w.data_ptr()), None))
    torch.cuda.synchronize()
    print(f"noalloc eigh N={n} batch {nb}: lowest eigenvalue {w.min().item():.2f}", flush=True)


def grad(nmol: int, nsamples: int, ntcf: int) -> None:
    """One loss + gradient evaluation (cir_loss_grad): the adjoint kernels."""
    p = cg.default_params(model="tip4p2005", species="H2O", ntcfpoints=ntcf, nsamples=nsamples, sampleEvery=2.0,
                          avef=3415.0, omegaStart=2000, omegaStop=5000, omegaStep=1)
    fos = cg.frame_table(p, 0.010)
    xyz, box = cg.synth_trajectory(nmol, int(fos.max()) + 1, seed=1)
    with cg.Engine(p, xyz.shape[1]) as eng:
        ref = eng.run(xyz, box, fos)
        L, g = eng.loss_grad(xyz, box, fos, 1.01 * ref["ls_ir"], 0.99 * ref["ls_vv"])
        print(f"grad nmol {nmol}: loss {L:.4e}", eng.stats(), flush=True)


def main() -> None:
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    e = sub.add_parser("eigh")
    e.add_argument("--nmol", type=int, default=512)
    e.add_argument("--batch", default="152")
    pr = sub.add_parser("prop")
    pr.add_argument("--n", type=int, default=1024)
    pr.add_argument("--nprop", type=int, default=10)
    pr.add_argument("--precision", default="fp32")
    r = sub.add_parser("run")
    r.add_argument("--nmol", type=int, default=512)
    r.add_argument("--nsamples", type=int, default=10)
    r.add_argument("--ntcf", type=int, default=250)
    r.add_argument("--precision", default="fp32")
    r.add_argument("--autotune", type=int, default=1)
    for opt in ("propagate-vectors", "share-frames", "refine-eigen"):
        r.add_argument("--" + opt, type=int, default=0)
    na = sub.add_parser("noalloc")
    na.add_argument("--nmol", type=int, default=256)
    na.add_argument("--batch", type=int, default=16)
    mu = sub.add_parser("multi")
    mu.add_argument("--sizes", default="128,216,343,512")
    mu.add_argument("--ntraj", type=int, default=4)
    mu.add_argument("--ntcf", type=int, default=200)
    sb = sub.add_parser("sbr")
    sb.add_argument("--nmol", type=int, default=512)
    sb.add_argument("--batch", type=int, default=2500)
    sb.add_argument("--reps", type=int, default=3)
    gr = sub.add_parser("grad")
    gr.add_argument("--nmol", type=int, default=256)
    gr.add_argument("--nsamples", type=int, default=2)
    gr.add_argument("--ntcf", type=int, default=32)
    a = ap.parse_args()
    if a.cmd == "eigh":
        eigh(a.nmol, [int(x) for x in a.batch.split(",")])
    elif a.cmd == "prop":
        prop(a.n, a.nprop, a.precision)
    elif a.cmd == "grad":
        grad(a.nmol, a.nsamples, a.ntcf)
    elif a.cmd == "multi":
        multi([int(x) for x in a.sizes.split(",")], a.ntraj, a.ntcf)
    elif a.cmd == "sbr":
        sbr(a.nmol, a.batch, a.reps)
    elif a.cmd == "noalloc":
        noalloc(a.nmol, a.batch)
    else:
        run(a.nmol, a.nsamples, a.ntcf, a.precision, propagate_vectors=a.propagate_vectors,
            share_frames=a.share_frames, refine_eigen=a.refine_eigen, autotune=a.autotune)


if __name__ == "__main__":
    main()
