"""CPU timing port of the reference's per-frame loop -- TEST/BENCH INFRASTRUCTURE ONLY.

The reference (calcIR.cu) has no CPU implementation of its hot path: every frame it
builds H on the GPU, calls MAGMA ssyevd, builds a dense propagator and multiplies three
complex matrices, then evaluates 15 complex gemv + dot pairs (calcIR.cu:404-745).  This
module restates that per-frame arithmetic on the host in FP32 / complex64 with numpy's
multithreaded LAPACK/BLAS (ssyevd, cgemm, cgemv), so bench.py can time the same algorithm
on the GPU machine's host cores as the reference-arm baseline.  Only bench.py's cpu_baseline
leg and its --impl reference arm may call it.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import oracle as O

HBAR = 5.308837367


def host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def frame_step(xyz, box, prm, state):
    """One frame-step of the reference algorithm (build, ssyevd, 3 cgemm, 15 gemv/dot)."""
    E, H, dip, pol = O.frame(xyz, box, prm)                        # calcIR.cu:404-406
    H32 = H.astype(np.float32)
    lam, V = np.linalg.eigh(H32)                                   # magma_ssyevd_gpu
    Vc = V.astype(np.complex64)
    m = np.vstack([dip, pol]).astype(np.complex64)
    if state.get("F") is None:                                     # k == 0: F = I
        state["F"] = np.eye(H.shape[0], dtype=np.complex64)
        state["m0"] = m
    else:
        P = np.diag(np.exp(1j * lam * np.float32(prm["dt"]) / HBAR).astype(np.complex64))   # Pinit
        T = Vc @ P                                                 # cgemm 1
        P2 = T @ Vc.T                                              # cgemm 2
        state["F"] = P2 @ state["F"]                               # cgemm 3 + ccopy
    F, m0 = state["F"], state["m0"]
    pairs = [(0, 0), (1, 1), (2, 2), (3, 3), (4, 4), (5, 5), (6, 6), (7, 7), (8, 8),
             (3, 4), (3, 5), (4, 3), (4, 5), (5, 3), (5, 4)]
    return [np.dot(m[b], F @ m0[a]) for a, b in pairs]             # 15 x (cgemv + cdotu)


def time_frame_steps(xyz_frames, box, prm, count: int) -> tuple[float, int]:
    """Seconds for `count` consecutive frame-steps of one origin and the thread count."""
    state = {}
    t = time.perf_counter()
    for k in range(count):
        frame_step(xyz_frames[k % len(xyz_frames)], box, prm, state)
    return time.perf_counter() - t, host_cores()
