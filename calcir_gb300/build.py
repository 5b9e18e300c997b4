"""Build recipe of the CUDA library and the drop-in executable, in tree.

Compiles every translation unit under ``csrc/`` for sm_103a (nvcc) or the host (g++)
in parallel and links ``libcalcir.so`` (the C ABI of ``include/calcir.h``) and the
``calcir`` executable next to this file.  Object files go to ``_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libcalcir.so")
EXE = os.path.join(HERE, "calcir")

CU = ["k_hamiltonian.cu", "k_eigh.cu", "k_dc.cu", "k_backtransform.cu", "k_adjoint.cu", "k_gemm.cu", "k_tc_gemm.cu", "k_tc_split.cu", "k_refine.cu", "k_tcf.cu", "k_fft.cu", "k_sbr.cu", "cir_api.cu"]
CPP = ["host_params.cpp", "host_synth.cpp", "host_traj.cpp", "host_xtc.cpp"]
MAIN = "calcir_main.cpp"
HEADERS = ["cir_device.cuh", "cir_internal.h", "cir_plan.h"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build calcir_gb300")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile what changed; returns the path of libcalcir.so."""
    nvcc = _nvcc()
    home = _cuda_home(nvcc)
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "calcir.h")]
    tasks = []
    objs = []
    for f in CU:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if _newer(obj, [src] + hdrs):
            # host code without FMA contraction: the same float results on x86-64 and aarch64
            tasks.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                          "-I" + INCLUDE, "-I" + CSRC, "-c", src, "-o", obj])
    for f in CPP + [MAIN]:
        src, obj = os.path.join(CSRC, f), os.path.join(BUILD, f + ".o")
        if f != MAIN:
            objs.append(obj)
        if _newer(obj, [src] + hdrs):
            # -ffp-contract=off keeps the synthetic generator bit-identical across CPUs
            tasks.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                          "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(home, "include"),
                          "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in tasks]:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            fut.result()
    if _newer(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    main_obj = os.path.join(BUILD, MAIN + ".o")
    if _newer(EXE, [main_obj, LIB]):
        _run([nvcc, *ARCH, "-o", EXE, main_obj, "-L" + HERE, "-lcalcir", "-lcudart",
              "-Xlinker", "-rpath=$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
