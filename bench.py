#!/usr/bin/env python
"""Throughput of the calcIR hot path on GB300: frame-steps per second.

A frame-step is one frame of one time origin: field + Hamiltonian build, eigensolve,
frequency distribution, propagation of F and the IR/Raman correlation contraction.
One bench step is one whole job of the full-size configuration: 512 rigid TIP4P/2005
molecules (1024 chromophores) in a 2.4834 nm box, 10 time origins 2 ps apart x 250
correlation points at 10 fs = 2500 frame-steps, on seeded synthetic frames.

  value  frame-steps/s with the positions already resident in HBM (cir_run on device
         pointers), device time by CUDA events on the library's stream
  e2e    the same through cir_run with pinned host buffers: positions copied in and all
         results copied out inside the timed region

--impl reference times the reference's per-frame algorithm (build, LAPACK dsyevd, three
complex GEMMs, 15 gemv/dot pairs) on the host cores, on the timed job's own frames and
origins, the only form of the reference that runs on the GPU machine (it needs MAGMA and
libxdrfile, which are not installed there).  That arm loads no compiled code of this
repository: its frames come from the numpy restatement of the generator.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "frames/s (H build+eig+propagate) @512 H2O, mixed vs FP32, ≤1e-3 spectrum err"
UNIT = "frames/s"
NMOL = 512
JOB = dict(model="tip4p2005", species="H2O", ntcfpoints=250, nsamples=10, sampleEvery=2.0, dt=0.010, t1=0.260,
           avef=3415.0, omegaStart=2000, omegaStop=5000, omegaStep=1, nzeros=25600, map=0)
WORKLOAD = ("512 TIP4P/2005 molecules (1024 chromophores, box 2.4834 nm), 10 time origins 2 ps apart x 250 "
            "correlation points at 10 fs = 2500 frame-steps per step")


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def job_roofline(n, fps, pk, precision):
    """The whole job against a time-weighted peak: W = 12.67 N^3 flops per frame-step (8 N^3
    propagation, 2 N^3 back-transform, 4/3 N^3 tridiagonalisation, 4/3 N^3 divide and conquer);
    in the mixed forms the propagation and back-transform on the tensor cores (BF16 peak / 3
    passes for split-BF16), the rest at the FP32 SIMT rate; in the plain form everything at
    the FP32 SIMT rate.  The SIMT rate is the nominal 152 SMs x 128 lanes x 2 flops x 2.07 GHz
    (80.5 TFLOP/s); the measured SGEMM rate is in peaks_probe."""
    simt = 152 * 128 * 2 * 2.07e9 / 1e12
    w_tc, w_simt = 10.0, 8.0 / 3.0
    if precision == "fp32":
        peak = simt
    else:
        tc = pk["bf16_tflops"] / (3.0 if precision == "bf16x3" else 2.0)
        peak = (w_tc + w_simt) / (w_tc / tc + w_simt / simt)
    achieved = 12.67 * n ** 3 * fps / 1e12
    return {"achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
            "work": "12.67 N^3 flops per frame-step (propagation 8, back-transform 2, tridiagonalisation 4/3, "
                    "divide and conquer 4/3)",
            "peak_kind": "time-weighted: tensor share at the measured BF16 peak / passes (TF32 at half the BF16 "
                         "rate), the rest at the nominal FP32 SIMT rate"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples every 200 ms during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.proc = None
        try:
            cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
            if gpu_id is not None:
                cmd += ["-i", str(gpu_id)]
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[4:8]):
                if v.lower() in ("active", "0x1") or v == "1":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def gpu_identifier():
    try:
        import torch
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        uuid = getattr(props, "uuid", None)
        if uuid:
            s = str(uuid)
            return s if s.startswith("GPU-") else "GPU-" + s
    except Exception:
        pass
    return None


# DRAM bytes (read + write) per 1024 x 1024 matrix of the tridiagonalisation kernel, from one
# ncu capture of k_eigh_tq on 152 matrices of order 1024 (dram__bytes_read.sum +
# dram__bytes_write.sum over the launch, / 152: 86.17 GB + 3.48 GB read and written, with
# the tiles of the matrix-vector products walked in alternating order):
#   python -m calcir_gb300.profile eigh --nmol 512 --batch 152 && \
#   ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum --clock-control none -k regex:k_eigh_tq -c 1 \
#       python -m calcir_gb300.profile eigh --nmol 512 --batch 152
TRIDIAG_DRAM_BYTES_PER_MATRIX = 0.590e9


def tridiag_bytes(n, nb=32):
    """Algorithmic DRAM bytes of the blocked tridiagonalisation of one order-n matrix: each
    column's matrix-vector product reads the lower triangle of its trailing block once, and
    each panel of nb columns reads and writes the lower triangle beyond the panel once."""
    sym = sum(4.0 * m * (m + 1) / 2 for m in range(1, n - 1))
    upd = sum(8.0 * (n - q0) * (n - q0 + 1) / 2 for q0 in range(nb, n - 1, nb))
    return sym + upd + 8.0 * 2 * 2   # + the final 2 x 2 block


PARITY_FIXTURE = os.path.join(ROOT, "tests", "golden", "fullsize_512h2o.npz")
PARITY_KEYS = ("tcf_ir", "tcf_vv", "tcf_vh", "ls_ir", "ls_vv", "ls_vh", "sw")


def parity(out, seed, bound, fixture=PARITY_FIXTURE):
    """Relative L2 error of each spectrum of a timed job against the FP64 oracle's spectra of
    the same job (512 H2O, 10 origins x 250 points, frames of seed 1; or the fixture given),
    stored as a fixture by tests/golden/make_fullsize.py."""
    if seed != 1 or not os.path.exists(fixture):
        return {"note": "no oracle fixture for this seed"}
    z = np.load(fixture)
    errs = {}
    for k in PARITY_KEYS:
        a, b = np.asarray(out[k]), z["fin_" + k]
        if a.shape != b.shape:
            return {"note": f"{k}: shape {a.shape} != fixture {b.shape}"}
        errs[k] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    return {"vs": f"FP64 oracle, the same job (tests/golden/{os.path.basename(fixture)})", "rel_l2": errs,
            "bound": bound, "within_bound": all(v < bound for v in errs.values())}


def make_frames(cg, seed):
    p = cg.default_params(**JOB)
    fos = cg.frame_table(p, 0.010)
    xyz, box = cg.synth_trajectory(NMOL, int(fos.max()) + 1, seed=seed)
    return p, xyz, box, fos


# the configuration both arms report (the reference arm times the same job's frame-steps)
CONFIG = {"workload": WORKLOAD, "nmol": NMOL, "nchrom": 2 * NMOL, "nsamples": JOB["nsamples"],
          "ntcfpoints": JOB["ntcfpoints"], "seed": 1,
          "l2": "no flush needed: each step streams ~20 GB of Hamiltonians and eigenvectors (>> 129 MB L2)"}
CPU_FORM = ("reference algorithm on the host cores (oracle/cpu_reference.py): build, LAPACK dsyevd in FP64 "
            "(scipy, evd driver), dense propagator + 3 complex64 cgemm, 15 cgemv/cdotu; frames from the numpy "
            "restatement of the seeded generator (oracle/synth.py)")


class CpuPort:
    """The reference algorithm on the host cores, on the frames of the timed job (seed 1 +
    rank): frames come from oracle/synth.py, which loads no compiled code of this
    repository.  One sample = the first `per` frame-steps of one time origin; successive
    samples walk the job's 10 origins."""

    def __init__(self, seed, per):
        from oracle import oracle as O
        from oracle import synth
        self.per = per
        self.prm = {"natom_mol": 4, "nchrom_mol": 2, "imodel": 1, "ispecies": 0, "map": JOB["map"],
                    "avef": JOB["avef"], "dt": JOB["dt"], "sampleEvery": JOB["sampleEvery"], "beginTime": 0.0}
        K = JOB["ntcfpoints"]
        self.tables = [[O.frame_index(self.prm, 0.010, s, k) for k in range(per)] for s in range(JOB["nsamples"])]
        nframes = max(t[-1] for t in self.tables) + 1
        assert per <= K
        self.xyz, self.box = synth.trajectory(NMOL, nframes, seed=seed)
        self.i = 0

    def sample(self):
        """(frame-steps per second, host threads) of the next sample."""
        from oracle import cpu_reference as R
        table = self.tables[self.i % len(self.tables)]
        self.i += 1
        sec, cores = R.time_origin(self.xyz, self.box, self.prm, table, self.per)
        return self.per / sec, cores


def run_reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    port = CpuPort(args.seed, args.cpu_sample)
    for _ in range(max(args.warmup, 0)):
        port.sample()
    rates, cores = [], 1
    for _ in range(args.steps):
        r, cores = port.sample()
        rates.append(r)
    value = float(len(rates) / np.sum(1.0 / np.asarray(rates)))     # total frame-steps / total seconds
    sample = (f"{args.cpu_sample} consecutive frame-steps (k = 0..{args.cpu_sample - 1}) of one time origin per "
              f"step, the steps walking the job's {JOB['nsamples']} origins; " + CPU_FORM)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": args.cpu_sample / value * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64 eig + c64 gemm",
            "data": "synthetic", "config": CONFIG, "form": "reference algorithm on the host CPU",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


BATCH_SIZES = (128, 216, 343, 512)
BATCH_JOB = dict(model="tip4p2005", species="H2O", ntcfpoints=200, nsamples=1, sampleEvery=2.0, dt=0.010, t1=0.260,
                 avef=3415.0, omegaStart=2000, omegaStop=5000, omegaStep=1, nzeros=25600, map=0)


def run_batching(args):
    """The batching configuration: 32 seeded trajectories of each of 128, 216, 343 and 512
    TIP4P/2005 molecules (256-1024 chromophores), 200 correlation points at 10 fs each, one
    time origin per trajectory, all in one cir_run_multi job (equal sizes batched through
    every launch, step loops replayed from captured CUDA graphs, SIMT tile shapes from the
    autotuner).  One bench step is the whole job; positions resident in HBM."""
    import torch
    torch.cuda.set_device(0)
    from calcir_gb300 import build
    build.build()
    import calcir_gb300 as cg
    stream = torch.cuda.current_stream()
    trajs, nsteps = [], 0
    for nmol in BATCH_SIZES:
        for t in range(args.batching_traj):
            xyz, box = cg.synth_trajectory(nmol, BATCH_JOB["ntcfpoints"], seed=args.seed * 1000 + nmol * 7 + t)
            d_xyz = torch.from_numpy(xyz).cuda()
            d_box = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(box, (xyz.shape[0], 3)))).cuda()
            trajs.append((d_xyz, d_box, None))
            nsteps += BATCH_JOB["ntcfpoints"]
    q = cg.default_params(**BATCH_JOB, precision=args.precision)
    warm = max(3, args.warmup)
    with cg.Engine(q, 4 * BATCH_SIZES[0]) as eng:
        eng.set_stream(stream.cuda_stream)
        for _ in range(warm):
            eng.run_multi(trajs)
        eng.reset_stats()
        torch.cuda.synchronize()
        sampler = ClockSampler(gpu_identifier())
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for _ in range(args.steps):
            eng.run_multi(trajs)
        t1.record(stream)
        torch.cuda.synchronize()
        clk = sampler.stop()
        ms = t0.elapsed_time(t1)
        st = eng.stats()
    line = {
        "metric": "frames/s, batching: uneven boxes 128/216/343/512 H2O x %d trajectories x 200 points" % args.batching_traj,
        "value": nsteps * args.steps / (ms * 1e-3), "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": warm,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else f"f32+{args.precision}", "data": "synthetic",
        "config": {"workload": f"{args.batching_traj} seeded trajectories of each of {list(BATCH_SIZES)} TIP4P/2005 "
                               "molecules, 200 correlation points at 10 fs, one origin each, one cir_run_multi job",
                   "frame_steps_per_step": nsteps, "cuda_graphs": True, "autotune": True},
        "stages_ms_per_step": {k: st[k] / args.steps for k in ("ms_build", "ms_eig", "ms_prop")},
        "gpu_launches": int(st["kernel_launches"]), "clocks": clk,
    }
    print(json.dumps(line), flush=True)


DIFF_JOB = dict(model="tip4p2005", species="H2O", ntcfpoints=200, nsamples=4, sampleEvery=2.0, dt=0.010, t1=0.260,
                avef=3415.0, omegaStart=2000, omegaStop=5000, omegaStep=1, nzeros=25600, map=0)


PRECISION_FIXTURE = os.path.join(ROOT, "tests", "golden", "fullsize_1024h2o.npz")


def run_precision(args):
    """The precision configuration: 1024 TIP4P/2005 molecules (2048 chromophores), 5 time
    origins 2 ps apart x 250 points = 1250 frame-steps per job, on seeded frames (seed 1).
    Each form -- the plain FP32 form and the mixed split-BF16 and TF32 forms -- is timed over
    --steps jobs after --warmup jobs, and its spectra are compared with the FP64 oracle's of
    the same job (bound 1e-4 for the plain form, 1e-3 for the mixed forms).  The line's value
    is the split-BF16 form's (the refinement option, about 46 ms per order-2048 matrix and
    step in FP64, is checked by the tests, not timed here)."""
    import torch
    torch.cuda.set_device(0)
    from calcir_gb300 import build
    build.build()
    import calcir_gb300 as cg
    job = dict(JOB, nsamples=5)
    p = cg.default_params(**job)
    fos = cg.frame_table(p, 0.010)
    xyz, box = cg.synth_trajectory(1024, int(fos.max()) + 1, seed=1)
    d_xyz = torch.from_numpy(xyz).cuda()
    d_box = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(box, (xyz.shape[0], 3)))).cuda()
    stream = torch.cuda.current_stream()
    steps, warm = max(1, args.steps), max(1, min(args.warmup, 2))
    forms = {}
    sampler = ClockSampler(gpu_identifier())
    for name, prec, bound in (("split-BF16", "bf16x3", 1e-3), ("TF32", "tf32", 1e-3), ("plain FP32", "fp32", 1e-4)):
        q = cg.default_params(**job, precision=prec)
        with cg.Engine(q, xyz.shape[1]) as eng:
            eng.set_stream(stream.cuda_stream)
            for _ in range(warm):
                eng.run(d_xyz.data_ptr(), d_box.data_ptr(), fos, nframes=xyz.shape[0])
            eng.reset_stats()
            torch.cuda.synchronize()
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(steps):
                out = eng.run(d_xyz.data_ptr(), d_box.data_ptr(), fos, nframes=xyz.shape[0])
            t1.record(stream)
            torch.cuda.synchronize()
            ms = t0.elapsed_time(t1)
            st = eng.stats()
        forms[name] = {"value": len(fos) * steps / (ms * 1e-3), "unit": "frame-steps/s", "ms_per_step": ms / steps,
                       "stages_ms_per_step": {k: st[k] / steps for k in ("ms_build", "ms_eig", "ms_prop")},
                       "parity": parity(out, 1, bound, PRECISION_FIXTURE)}
    clk = sampler.stop()
    head = forms["split-BF16"]
    line = {
        "metric": "frame-steps/s, precision: 1024 H2O (2048 chromophores), 5 origins x 250 points",
        "value": head["value"], "unit": "frame-steps/s", "n_gpus": 1, "steps": steps, "warmup": warm,
        "ms_per_step": head["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+bf16x3", "data": "synthetic",
        "config": {"workload": "1024 TIP4P/2005 molecules (2048 chromophores), 5 time origins 2 ps apart x 250 "
                               "correlation points at 10 fs = 1250 frame-steps per step", "seed": 1},
        "forms": forms,
        "mixed_over_plain": head["value"] / forms["plain FP32"]["value"],
        "clocks": clk,
    }
    print(json.dumps(line))
    return 0


def run_differentiation(args):
    """The differentiation configuration: 256 TIP4P/2005 molecules (512 chromophores), 4 time
    origins x 200 points; the loss is the IR + VV lineshape mismatch against targets made by
    the same code with the map coefficients perturbed by seeded +-2% noise.  One bench step is
    one loss + gradient evaluation (cir_loss_grad: forward, psi checkpoints every 16 steps,
    adjoint backward).  The gradient is checked against GPU central differences (relative
    step 1e-4) on the three coefficients the loss is most sensitive to."""
    import torch
    torch.cuda.set_device(0)
    from calcir_gb300 import build
    build.build()
    import calcir_gb300 as cg
    q = cg.default_params(**DIFF_JOB)
    fos = cg.frame_table(q, 0.010)
    xyz, box = cg.synth_trajectory(256, int(fos.max()) + 1, seed=args.seed)
    stream = torch.cuda.current_stream()
    with cg.Engine(q, xyz.shape[1]) as eng:
        eng.set_stream(stream.cuda_stream)
        th0 = eng.get_coeffs().astype(np.float64)
        tht = th0 * (1 + 0.02 * np.random.default_rng(args.seed).uniform(-1, 1, 13))
        eng.set_coeffs(tht.astype(np.float32))
        ref = eng.run(xyz, box, fos)
        targets = (ref["ls_ir"].astype(np.float32), ref["ls_vv"].astype(np.float32))
        eng.set_coeffs(th0.astype(np.float32))
        warm = max(3, args.warmup)
        for _ in range(warm):
            eng.loss_grad(xyz, box, fos, *targets)
        eng.reset_stats()
        torch.cuda.synchronize()
        sampler = ClockSampler(gpu_identifier())
        t0 = time.perf_counter()
        for _ in range(args.steps):
            L, g = eng.loss_grad(xyz, box, fos, *targets)
        torch.cuda.synchronize()
        sec = (time.perf_counter() - t0) / args.steps
        clk = sampler.stop()
        st = eng.stats()
        sens = np.abs(g * th0)
        checks = []
        for qi in np.argsort(-sens)[:3]:
            h = 1e-4 * abs(th0[qi])
            lv = []
            for sgn in (1, -1):
                t = th0.copy()
                t[qi] += sgn * h
                eng.set_coeffs(t.astype(np.float32))
                lv.append(eng.loss_grad(xyz, box, fos, *targets)[0])
            step = float(np.float32(th0[qi] + h)) - float(np.float32(th0[qi] - h))
            fd = (lv[0] - lv[1]) / step
            checks.append({"coefficient": ["w0", "w1", "w2", "x0", "x1", "p0", "p1", "mup0", "mup1", "mup2", "wi0",
                                           "wi1", "wi2"][qi], "adjoint": float(g[qi]), "central_difference": fd,
                           "rel_diff": abs(fd - g[qi]) / abs(g[qi])})
        eng.set_coeffs(th0.astype(np.float32))
    nsteps = len(fos)
    line = {
        "metric": "frame-steps/s of loss + adjoint gradient, differentiation: 256 H2O, 4 origins x 200 points",
        "value": nsteps / sec, "unit": "frame-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": warm,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "256 TIP4P/2005 molecules (512 chromophores), 4 origins 2 ps apart x 200 points; "
                               "targets from map coefficients perturbed by seeded +-2% noise; psi checkpoints every "
                               "16 steps", "loss": L},
        "gradient_checks": checks, "gpu_launches": int(st["kernel_launches"]), "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="bf16x3", choices=["fp32", "tf32", "bf16x3"],
                    help="arithmetic of the propagation GEMMs for the headline number")
    ap.add_argument("--no-plain", action="store_true", help="skip timing the plain FP32 form and the run options beside it")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-sample", type=int, default=8, help="frame-steps per CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="full", choices=["full", "batching", "differentiation", "precision"],
                    help="full: the 512 H2O job (the headline); batching: uneven boxes of 128/216/343/512 "
                         "molecules, --batching-traj trajectories of each size, in one cir_run_multi job; "
                         "differentiation: loss + gradient at 256 H2O; precision: 1024 H2O, 5 x 250, each form")
    ap.add_argument("--batching-traj", type=int, default=32)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "batching":
        return run_batching(args)
    if args.workload == "differentiation":
        return run_differentiation(args)
    if args.workload == "precision":
        return run_precision(args)

    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from calcir_gb300 import build
    build.build()
    import calcir_gb300 as cg

    # weak scaling: every rank runs its own 10-origin job on its own seeded trajectory
    p, xyz, box, fos = make_frames(cg, args.seed + rank)
    steps_per_job = len(fos)
    stream = torch.cuda.current_stream()
    d_xyz = torch.from_numpy(xyz).cuda()
    d_box = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(box, (xyz.shape[0], 3)))).cuda()
    h_xyz = torch.from_numpy(xyz).pin_memory()
    h_box = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(box, (xyz.shape[0], 3)))).pin_memory()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def time_form(precision, steps, warmup, e2e=True, clocks=False, **opts):
        """(device ms, e2e ms, stats, clock record) of `steps` jobs after `warmup` jobs."""
        q = cg.default_params(**JOB, precision=precision, **opts)
        res = {}
        with cg.Engine(q, xyz.shape[1]) as eng:
            eng.set_stream(stream.cuda_stream)
            for _ in range(warmup):
                eng.run(d_xyz.data_ptr(), d_box.data_ptr(), fos, nframes=xyz.shape[0])
            eng.reset_stats()
            torch.cuda.synchronize()
            barrier()
            sampler = ClockSampler(gpu_identifier()) if clocks else None
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            for _ in range(steps):
                out = eng.run(d_xyz.data_ptr(), d_box.data_ptr(), fos, nframes=xyz.shape[0])
            t1.record(stream)
            torch.cuda.synchronize()
            barrier()
            res["clk"] = sampler.stop() if sampler else None
            res["ms"] = t0.elapsed_time(t1)
            res["out"] = out
            res["stats"] = eng.stats()
            if e2e:
                torch.cuda.synchronize()
                barrier()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(steps):
                    eng.run(h_xyz.data_ptr(), h_box.data_ptr(), fos, nframes=xyz.shape[0])
                e1.record(stream)
                torch.cuda.synchronize()
                barrier()
                res["ms_e2e"] = e0.elapsed_time(e1)
        return res

    warm = max(args.warmup, 3)
    main_res = time_form(args.precision, args.steps, warm, e2e=True, clocks=True)
    plain = None
    if args.precision != "fp32" and not args.no_plain:
        plain = time_form("fp32", args.steps, warm, e2e=False)
    # the options that reach the same results with less work, timed separately (never the headline)
    options = {}
    if not args.no_plain:
        for name, opts in (("share_frames", {"share_frames": 1}),
                           ("propagate_vectors", {"propagate_vectors": 1}),
                           ("share_frames+propagate_vectors", {"share_frames": 1, "propagate_vectors": 1})):
            r = time_form(args.precision, args.steps, 2, e2e=False, **opts)
            options[name] = {"value": steps_per_job * args.steps / (r["ms"] * 1e-3), "unit": UNIT,
                             "eigensolves_per_job": r["stats"]["eig_matrices"] // args.steps,
                             "stages_ms_per_step": {k: r["stats"][k] / args.steps for k in ("ms_build", "ms_eig", "ms_prop")}}
    ms, ms_e2e, st, clk = main_res["ms"], main_res["ms_e2e"], main_res["stats"], main_res["clk"]

    if world > 1:
        t = torch.tensor([ms, ms_e2e], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms, ms_e2e = t.tolist()
    total_steps = steps_per_job * args.steps * world
    value = total_steps / (ms * 1e-3)
    e2e = total_steps / (ms_e2e * 1e-3)

    n = NMOL * 2
    pk, pk_kind = peaks()
    eig_ms_per_launch = st["ms_eig"] / args.steps          # one eigensolver launch sequence per job (one chunk)
    eig_flops = 10.0 / 3.0 * n ** 3 * steps_per_job         # nominal eigensolver flops per job
    eig_tflops = eig_flops / (eig_ms_per_launch * 1e-3) / 1e12
    tq_ms = st["ms_tridiag"] / args.steps                  # the job's tridiagonalisation: end of the build to the
                                                           # end of the later of its two launches (two streams)
    tq_bytes = tridiag_bytes(n) * steps_per_job
    tq_gbs = tq_bytes / (tq_ms * 1e-3) / 1e9
    prop_flops = 8.0 * n ** 3 * JOB["nsamples"] * (JOB["ntcfpoints"] - 1)
    prop_tflops = prop_flops / (st["ms_prop"] / args.steps * 1e-3) / 1e12
    passes = {"fp32": 1, "tf32": 1, "bf16x3": 3}[args.precision]   # tensor-pipe passes per product
    nfft = JOB["ntcfpoints"] + JOB["nzeros"]
    nomega = 3001
    h2d = xyz.nbytes + xyz.shape[0] * 12 + fos.nbytes
    d2h = steps_per_job * 48 + nomega * 8 * 4 + 3 * nfft * 8
    form = {"fp32": "plain FP32 (SIMT GEMMs)", "tf32": "mixed: TF32 tcgen05 propagation GEMMs",
            "bf16x3": "mixed: 3-pass split-BF16 tcgen05 propagation GEMMs"}[args.precision]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": warm, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if args.precision == "fp32" else f"f32+{args.precision}",
        "data": "synthetic",
        "config": CONFIG, "form": form,
        "stages_ms_per_step": {k: st[k] / args.steps for k in ("ms_build", "ms_eig", "ms_prop")},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(st["kernel_launches"]),
        "roofline": {"kernel": "k_eigh_tq (blocked lower-storage tridiagonalisation; the job's 2500 matrices in "
                               "two launches on two streams, timed together)",
                     "bound": "hbm", "achieved": tq_gbs, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": tq_gbs / pk["hbm_gbs"], "peak_kind": f"{pk_kind} copy bandwidth (burst)",
                     "work": "algorithmic bytes: per column the lower triangle of the trailing block, per "
                             "32-column panel one read and write of the trailing lower triangle; "
                             f"{tridiag_bytes(n) / 1e9:.3f} GB per 1024 x 1024 matrix x 2500 matrices per job",
                     "ms_per_launch": tq_ms,
                     "traffic": TRIDIAG_DRAM_BYTES_PER_MATRIX * steps_per_job,
                     "traffic_note": "ncu dram__bytes_read.sum + dram__bytes_write.sum per matrix x 2500"},
        "roofline_eigensolver": {"kernels": "tridiagonalisation, divide and conquer, blocked Householder "
                                            "back-transform V = Q_H Q_T",
                                 "achieved": eig_tflops, "unit": "TFLOP/s",
                                 "work": "10/3 N^3 nominal flops per matrix (4/3 N^3 tridiagonalisation + 2 N^3 "
                                         "back-transform; merge products not counted) x 2500 matrices"},
        "roofline_propagation": {"kernel": f"propagation GEMMs ({args.precision})", "bound": "tensor",
                                 "achieved": prop_tflops * passes, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                                 "frac": prop_tflops * passes / pk["bf16_tflops"],
                                 "algorithmic_tflops": prop_tflops,
                                 "work": f"{8 * passes} N^3 tensor-pipe flops per origin-step ({passes} pass(es) of "
                                         "the two real N x 2N x N GEMMs, 8 N^3 algorithmic), 10 origins x 249 steps; "
                                         "time includes the V split and the correlation contraction"},
        "roofline_job": job_roofline(n, value, pk, args.precision),
        "clocks": clk,
    }
    if options:
        line["options"] = dict(options, note="same results by less work (frame sharing across the overlapping "
                                             "origins; propagating psi = F m(0) instead of F), reported beside the "
                                             "headline, which does the reference's full work")
    line["parity"] = parity(main_res["out"], args.seed + rank, 1e-4 if args.precision == "fp32" else 1e-3)
    if plain is not None:
        line["plain_fp32"] = {"parity": parity(plain["out"], args.seed + rank, 1e-4),"value": total_steps / (plain["ms"] * 1e-3) / world * world, "unit": UNIT,
                              "ms_per_step": plain["ms"] / args.steps,
                              "stages_ms_per_step": {k: plain["stats"][k] / args.steps for k in ("ms_build", "ms_eig", "ms_prop")},
                              "mixed_over_plain": plain["ms"] / ms}
    if rank == 0:
        # FP32-SIMT / TF32 / FP64 cuBLAS peaks (not in the peak file), measured after the timed
        # regions: the denominators of the plain form's SIMT propagation roofline
        try:
            from calcir_gb300 import peaks as peak_probe
            extra = peak_probe.measure(quick=True)
        except Exception as exc:        # a probe failure must not lose the bench line
            extra = {"error": f"{type(exc).__name__}: {exc}"}
        line["peaks_probe"] = extra
        if plain is not None and "fp32_simt_tflops" in extra:
            plain_prop = prop_flops / (plain["stats"]["ms_prop"] / args.steps * 1e-3) / 1e12
            line["plain_fp32"]["roofline_propagation"] = {
                "kernel": "k_sgemm (SIMT FP32 propagation GEMMs)", "bound": "fp32 simt", "achieved": plain_prop,
                "peak": extra["fp32_simt_tflops"], "unit": "TFLOP/s", "frac": plain_prop / extra["fp32_simt_tflops"],
                "peak_kind": "measured cuBLAS SGEMM, TF32 off (peaks_probe)"}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        port = CpuPort(args.seed, args.cpu_sample)
        port.sample()                                   # warm-up (threads, page faults)
        got = [port.sample() for _ in range(2)]
        rates = np.asarray([r for r, _ in got])
        line["cpu_baseline"] = {"value": float(2 / np.sum(1.0 / rates)), "unit": UNIT,
                                "cores": got[-1][1], "kind": "port",
                                "sample": f"2 x {args.cpu_sample} frame-steps (origins 1 and 2 of the job); "
                                          + CPU_FORM}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
