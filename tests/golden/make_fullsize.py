"""Makes the full-length FP64 oracle fixtures of the two large water configurations.

TEST INFRASTRUCTURE.  The oracle (oracle/oracle.py, FP64, psi-vector propagation) runs the
whole job of each configuration on seeded synthetic frames and the raw sums are stored:

  fullsize_512h2o.npz   512 TIP4P/2005 molecules (1024 chromophores), 10 time origins 2 ps
                        apart x 250 correlation points (2500 frame-steps), seed 1 -- the
                        frames and parameters of bench.py's timed job
  fullsize_1024h2o.npz  1024 molecules (2048 chromophores), 5 origins x 250 points, seed 1

Each fixture holds the raw correlation sums per step (complex, 3 x 250), the spectral
density and the frequency-distribution sums (3001 bins each) and the job parameters, and
the finished spectra that oracle.finish makes of them (damped correlation functions,
spectral density, and the three lineshapes in float32), so that bench.py can state the
error of its timed run without running any oracle code; a few hundred KB each.  The frames come from the
project's seeded generator (bit-identical on x86-64 and aarch64, and to the numpy
restatement in oracle/synth.py); the time origins run in parallel worker processes, one
origin each, and their sums are added (oracle.merge).

Usage: python tests/golden/make_fullsize.py [512|1024 ...] [--workers W]
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

CONFIGS = {
    512: dict(nmol=512, seed=1, nsamples=10, name="fullsize_512h2o"),
    1024: dict(nmol=1024, seed=1, nsamples=5, name="fullsize_1024h2o"),
}
# bench.py's job (input.inp keys): map 0, H2O, tip4p2005 (imodel 1)
JOB = dict(ntcfpoints=250, sampleEvery=2.0, dt=0.010, t1=0.260, avef=3415.0, omegaStart=2000, omegaStop=5000,
           omegaStep=1, nzeros=25600, map=0, beginTime=0.0, natom_mol=4, nchrom_mol=2, imodel=1, ispecies=0)
FRAME_DT = 0.010


def oracle_params(nsamples: int) -> dict:
    return dict(JOB, nsamples=nsamples)


def frame_table(prm: dict) -> np.ndarray:
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    return np.array([O.frame_index(prm, FRAME_DT, s, k) for s in range(prm["nsamples"])
                     for k in range(prm["ntcfpoints"])], np.int64)


def _worker(args):
    prm, s, frames, box = args
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    # frames holds only this origin's frames; remap the table to them
    K = prm["ntcfpoints"]
    table = np.zeros(prm["nsamples"] * K, np.int64)
    table[s * K:(s + 1) * K] = np.arange(K)
    t = time.time()
    acc = O.accumulate(prm, frames, [box] * len(frames), table, samples=[s])
    return s, acc, time.time() - t


def make(nmol_key: int, workers: int) -> str:
    sys.path.insert(0, ROOT)
    import calcir_gb300 as cg
    from oracle import oracle as O
    cfg = CONFIGS[nmol_key]
    prm = oracle_params(cfg["nsamples"])
    fos = frame_table(prm)
    xyz, box = cg.synth_trajectory(cfg["nmol"], int(fos.max()) + 1, seed=cfg["seed"])
    K = prm["ntcfpoints"]
    tasks = [(prm, s, np.ascontiguousarray(xyz[fos[s * K:(s + 1) * K]]), box) for s in range(prm["nsamples"])]
    # one LAPACK thread per worker process: the workers inherit this environment
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"
    ctx = mp.get_context("spawn")
    t0 = time.time()
    with ctx.Pool(workers) as pool:
        parts = []
        for s, acc, sec in pool.imap_unordered(_worker, tasks):
            print(f"{cfg['name']}: origin {s} done in {sec:.0f} s", flush=True)
            parts.append((s, acc))
    parts.sort(key=lambda x: x[0])
    acc = O.merge([a for _, a in parts])
    out = os.path.join(HERE, cfg["name"] + ".npz")
    save(out, cfg, prm, fos, acc)
    print(f"wrote {out} ({time.time() - t0:.0f} s)", flush=True)
    return out


def save(out, cfg, prm, fos, acc):
    sys.path.insert(0, ROOT)
    from oracle import oracle as O
    fin = O.finish(prm, acc)
    np.savez_compressed(out, tcf=acc["tcf"], sw=acc["sw"], count=acc["count"], ipr=acc["ipr"], mipr=acc["mipr"],
                        oor=acc["oor"], nchrom=acc["nchrom"], omega=acc["omega"], nmol=cfg["nmol"],
                        seed=cfg["seed"], nsamples=cfg["nsamples"], frame_table=fos,
                        job=np.array(repr(sorted(prm.items()))),
                        fin_tcf_ir=fin["tcf_ir"], fin_tcf_vv=fin["tcf_vv"], fin_tcf_vh=fin["tcf_vh"], fin_sw=fin["sw"],
                        fin_ls_ir=fin["ls_ir"].astype(np.float32), fin_ls_vv=fin["ls_vv"].astype(np.float32),
                        fin_ls_vh=fin["ls_vh"].astype(np.float32), fin_ls_len=len(fin["ls_omega"]))


def refinish(nmol_key: int) -> None:
    """Rewrites a fixture's finished spectra from its raw sums."""
    cfg = CONFIGS[nmol_key]
    path = os.path.join(HERE, cfg["name"] + ".npz")
    prm, acc, _, _, fos = load(path)
    save(path, cfg, prm, fos, acc)


def load(path: str):
    """(oracle parameters, raw sums) of a fixture, ready for oracle.finish."""
    z = np.load(path)
    prm = oracle_params(int(z["nsamples"]))
    acc = {k: z[k] for k in ("tcf", "sw", "count", "ipr", "mipr", "omega")}
    acc["oor"] = int(z["oor"])
    acc["nchrom"] = int(z["nchrom"])
    return prm, acc, int(z["nmol"]), int(z["seed"]), z["frame_table"]


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("sizes", nargs="*", type=int, default=[512, 1024])
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--refinish", action="store_true", help="only recompute the finished spectra")
    a = ap.parse_args()
    for n in a.sizes:
        refinish(n) if a.refinish else make(n, a.workers)
