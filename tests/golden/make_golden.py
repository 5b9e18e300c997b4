"""Generate the golden fixtures of tests/golden from the reference program itself.

The reference (nicholashestand/calcIR, ``calcIR.cu``) is built for the host CPU from its
own sources by ``oracle/build_ref.sh`` (shim headers stand in for MAGMA, libxdrfile and
cuFFT).  For every case below this script writes a seeded synthetic trajectory
(CIRTRJ01) and an input.inp, runs ``oracle/_ref/calcIR_ref input.inp``, and stores the
13 output files it writes as arrays in ``<case>.npz`` together with the parameters in
``<case>.json``.  Parser cases run the reference on tricky input files and keep the
parameter lines it prints (calcIR.cu:70-87).

Run from the repository root (needs the reference sources and libcalcir.so):
    python tests/golden/make_golden.py [reference_dir]
The reference directory is the argument, else $CALCIR_REFERENCE_DIR, else the default of
oracle/build_ref.sh.  Each run works in a fresh temporary directory.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import calcir_gb300 as cg  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")
WORK = None   # set by main(): a fresh temporary directory per run

# (case name, synthetic nmol, seed, input keys); frame_dt of every trajectory is 0.010 ps
CASES = [
    ("small_h2o", 64, 11, dict(model="tip4p2005", species="H2O", map=0, ntcfpoints=150, nsamples=1,
                              sampleEvery=10.0, dt=0.010, t1=0.260, avef=3415.0, omegaStart=2000,
                              omegaStop=5000, omegaStep=1, nzeros=25600, beginTime=0)),
    ("multi_d2o_map1", 32, 5, dict(model="e3b2", species="D2O", map=1, ntcfpoints=40, nsamples=3,
                                   sampleEvery=0.2, dt=0.020, t1=0.200, avef=2500.0, omegaStart=500,
                                   omegaStop=3500, omegaStep=5, nzeros=2000, beginTime=0.1)),
    ("hod_d2o", 32, 7, dict(model="tip4p2005", species="HOD/D2O", map=0, ntcfpoints=30, nsamples=2,
                            sampleEvery=0.3, dt=0.010, t1=0.260, avef=3400.0, omegaStart=1000,
                            omegaStop=5000, omegaStep=2, nzeros=500, beginTime=0)),
    ("bend_hod_h2o", 24, 3, dict(model="e3b3", species="HOD/H2O", map=1, ntcfpoints=20, nsamples=1,
                                 sampleEvery=1.0, dt=0.010, t1=0.300, avef=2600.0, omegaStart=1000,
                                 omegaStop=4000, omegaStep=3, nzeros=300, beginTime=0.05, nchrom_mol=1)),
]

PARSER_CASES = {
    "parse_basic": "xtcf nope.xtc // comment\noutf p1\nntcfpoints 77\nnsamples 3\nsampleEvery 2.5\n"
                   "omegaStep 4\nmap 1\nspecies D2O\nmodel tip4p\ndt 0.02\nt1 0.3\navef 3300.5\n"
                   "omegaStart 1800\nomegaStop 4200\nnzeros 1234\nbeginTime 1.5\n",
    "parse_quirks": "#avef 2415.2 // commented-out key warns\nxtcf\nnope2.xtc extra tokens here\n"
                    "ntcfpoints 12.9\nnsamples abc\nomegaStep 7 more\nbogus 5\navef 1e3\n"
                    "species HOD/H2O\nnzeros -3\noutf p2\n",
}

FILES = ["irrtcf", "iritcf", "vvrtcf", "vvitcf", "vhrtcf", "vhitcf", "spdn", "Pw", "Rw", "Rmw",
         "irls", "vvls", "vhls"]


def input_text(keys: dict, xtcf: str, outf: str) -> str:
    lines = [f"xtcf {xtcf}", f"outf {outf}", "natom_mol 4"]
    lines += [f"{k} {v}" for k, v in keys.items()]
    return "\n".join(lines) + "\n"


def frames_needed(keys: dict) -> int:
    p = cg.default_params(**{k: v for k, v in keys.items() if k not in ("model", "species")},
                          model=keys["model"], species=keys["species"])
    return int(cg.frame_table(p, 0.010).max()) + 1


def run_case(exe: str, name: str, nmol: int, seed: int, keys: dict) -> None:
    d = os.path.join(WORK, name)
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    nfr = frames_needed(keys) + 2
    xyz, box = cg.synth_trajectory(nmol, nfr, seed=seed)
    cg.write_traj(os.path.join(d, "traj.cirtrj"), xyz, box, 0.010)
    with open(os.path.join(d, "input.inp"), "w") as f:
        f.write(input_text(keys, "traj.cirtrj", "ref"))
    r = subprocess.run([exe, "input.inp"], cwd=d, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{name}: reference failed\n{r.stdout[-2000:]}")
    if "bin_num" in r.stdout:
        # the reference then writes outside its histogram arrays (calcIR.cu:529-537)
        raise RuntimeError(f"{name}: eigenvalues outside [omegaStart, omegaStop]; widen the window")
    arrays = {}
    for fn in FILES:
        a = np.loadtxt(os.path.join(d, f"ref_{fn}.dat"), ndmin=2)
        arrays[fn] = a.astype(np.float64)
    with open(os.path.join(d, "ref_irrtcf.dat")) as f:
        arrays["irrtcf_text_head"] = np.frombuffer(f.read(400).encode(), np.uint8)
    np.savez_compressed(os.path.join(GOLDEN, f"{name}.npz"), **arrays)
    meta = {"nmol": nmol, "seed": seed, "frame_dt": 0.010, "nframes": nfr, "keys": keys,
            "warnings": [ln for ln in r.stdout.splitlines() if "WARNING" in ln]}
    with open(os.path.join(GOLDEN, f"{name}.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)
    print(name, "ok", {k: v.shape for k, v in arrays.items()})


def run_parser_case(exe: str, name: str, text: str) -> None:
    d = os.path.join(WORK, name)
    shutil.rmtree(d, ignore_errors=True)
    os.makedirs(d)
    with open(os.path.join(d, "input.inp"), "w") as f:
        f.write(text)
    r = subprocess.run([exe, "input.inp"], cwd=d, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("\tSetting") or "WARNING" in ln]
    with open(os.path.join(GOLDEN, f"{name}.json"), "w") as f:
        json.dump({"input": text, "stdout": lines, "returncode": r.returncode}, f, indent=1)
    print(name, "ok", len(lines), "lines")


def main() -> None:
    global WORK
    ref_dir = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CALCIR_REFERENCE_DIR")
    cmd = [os.path.join(ROOT, "oracle", "build_ref.sh")] + ([ref_dir] if ref_dir else [])
    exe = subprocess.run(cmd, check=True, stdout=subprocess.PIPE, text=True).stdout.strip().splitlines()[-1]
    WORK = tempfile.mkdtemp(prefix="calcir_golden_")
    for name, nmol, seed, keys in CASES:
        run_case(exe, name, nmol, seed, keys)
    for name, text in PARSER_CASES.items():
        run_parser_case(exe, name, text)


if __name__ == "__main__":
    main()
