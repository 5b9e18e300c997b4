"""Makes the FP64 oracle fixtures of the batching and differentiation configurations.

TEST INFRASTRUCTURE.

  batching_2traj.npz  uneven boxes of 128, 216, 343 and 512 TIP4P/2005 molecules (256-1024
                      chromophores), 2 seeded trajectories of each size (seeds 1000 + 7 nmol
                      + t, the seeds bench.py's batching workload gives its first two
                      trajectories of each size), 200 correlation points at 10 fs, one time
                      origin each: per trajectory the raw correlation and spectral-density
                      sums of oracle.accumulate (batching_spectra finishes them)
  diff_256h2o.npz     256 molecules (512 chromophores), 4 origins 2 ps apart x 200 points,
                      frames of seed 1: target IR and VV lineshapes made by the FP64 forward
                      pass with the map coefficients perturbed by seeded +-2% noise (rounded
                      to float32, as the GPU form takes them), and at the unperturbed
                      coefficients the loss and its gradient by the FP64 adjoint
                      (oracle/adjoint.py, which matches FP64 central differences)

Usage: python tests/golden/make_configs.py [batching] [differentiation] [--workers W]
"""
from __future__ import annotations

import argparse
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

BATCH_SIZES = (128, 216, 343, 512)
BATCH_TRAJ = 2
BATCH_PRM = dict(ntcfpoints=200, nsamples=1, sampleEvery=2.0, dt=0.010, t1=0.260, avef=3415.0, omegaStart=2000,
                 omegaStop=5000, omegaStep=1, nzeros=25600, map=0, beginTime=0.0, natom_mol=4, nchrom_mol=2,
                 imodel=1, ispecies=0)
DIFF_PRM = dict(BATCH_PRM, nsamples=4)
DIFF_NMOL, DIFF_SEED, DIFF_NOISE_SEED = 256, 1, 1
FRAME_DT = 0.010


def batch_seed(nmol: int, t: int) -> int:
    return 1000 + nmol * 7 + t


def _batch_worker(args):
    nmol, t = args
    sys.path.insert(0, ROOT)
    import calcir_gb300 as cg
    from oracle import oracle as O
    xyz, box = cg.synth_trajectory(nmol, BATCH_PRM["ntcfpoints"], seed=batch_seed(nmol, t))
    tm = time.time()
    acc = O.accumulate(BATCH_PRM, xyz, [box] * len(xyz), np.arange(BATCH_PRM["ntcfpoints"]))
    return nmol, t, acc, time.time() - tm


def make_batching(workers: int) -> None:
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"
    tasks = [(n, t) for n in reversed(BATCH_SIZES) for t in range(BATCH_TRAJ)]
    out = {}
    with mp.get_context("spawn").Pool(workers) as pool:
        for nmol, t, acc, sec in pool.imap_unordered(_batch_worker, tasks):
            print(f"batching {nmol} H2O trajectory {t}: {sec:.0f} s", flush=True)
            key = f"n{nmol}_t{t}_"
            for k in ("tcf", "sw", "oor", "nchrom"):
                out[key + k] = acc[k]
    np.savez_compressed(os.path.join(HERE, "batching_2traj.npz"), **out)
    print("wrote batching_2traj.npz", flush=True)


def batching_spectra(z, key):
    """Correlation functions, spectral density and lineshapes of one trajectory of the
    batching fixture (its raw correlation and spectral-density sums, finished by the oracle)."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    nom = O.nomega(BATCH_PRM)
    acc = {"tcf": z[key + "tcf"], "sw": z[key + "sw"], "oor": int(z[key + "oor"]), "nchrom": int(z[key + "nchrom"]),
           "count": np.ones(nom), "ipr": np.zeros(nom), "mipr": np.zeros(nom), "omega": np.zeros(nom)}
    return O.finish(BATCH_PRM, acc)


def diff_frames(lib_synth):
    """(frames, box, frame table) of the differentiation configuration."""
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    fos = np.array([O.frame_index(DIFF_PRM, FRAME_DT, s, k) for s in range(DIFF_PRM["nsamples"])
                    for k in range(DIFF_PRM["ntcfpoints"])], np.int64)
    xyz, box = lib_synth(DIFF_NMOL, int(fos.max()) + 1, seed=DIFF_SEED)
    return xyz, box, fos


def perturbed_theta():
    sys.path.insert(0, ROOT)
    from oracle import adjoint as A
    from oracle import oracle as O
    th0 = A.theta_of(O.maps(0, 0))
    noise = np.random.default_rng(DIFF_NOISE_SEED).uniform(-1, 1, 13)
    return th0, (th0 * (1 + 0.02 * noise)).astype(np.float32).astype(np.float64)


def make_differentiation() -> None:
    sys.path.insert(0, ROOT)
    import calcir_gb300 as cg
    from oracle import adjoint as A
    xyz, box, fos = diff_frames(cg.synth_trajectory)
    boxes = [box] * len(xyz)
    th0, tht = perturbed_theta()
    t0 = time.time()
    tir, tvv, _ = A.forward(DIFF_PRM, tht, xyz, boxes, fos)
    targets = [t.astype(np.float32) for t in A.lineshapes(DIFF_PRM, tir, tvv)]
    print(f"targets: {time.time() - t0:.0f} s", flush=True)
    t64 = [t.astype(np.float64) for t in targets]
    L, g = A.adjoint_grad(DIFF_PRM, th0, xyz, boxes, fos, t64)
    print(f"loss {L:.6e}, gradient by the adjoint: {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(os.path.join(HERE, "diff_256h2o.npz"), target_ir=targets[0], target_vv=targets[1],
                        theta0=th0, theta_target=tht, loss=L, grad=np.asarray(g, np.float64), frame_table=fos)
    print("wrote diff_256h2o.npz", flush=True)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("what", nargs="*", default=["batching", "differentiation"])
    ap.add_argument("--workers", type=int, default=3)
    a = ap.parse_args()
    if "batching" in a.what:
        make_batching(a.workers)
    if "differentiation" in a.what:
        make_differentiation()
