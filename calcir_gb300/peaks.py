"""Arithmetic peaks that MEASURED_PEAKS.json (HBM copy and BF16 GEMM) does not hold: FP32 on the SIMT pipe
(cuBLAS SGEMM with TF32 off), TF32 on the tensor cores and FP64, each as the best of a few
back-to-back cuBLAS GEMMs timed with CUDA events.  They are the denominators of the plain
form's FP32 rooflines (SIMT propagation GEMMs, merge and back-transform products) and of the
opt-in FP64 eigenpair refinement.

    python -m calcir_gb300.peaks            # one JSON line
"""
from __future__ import annotations

import json

import torch


def _gemm_tflops(dtype: torch.dtype, n: int, reps: int, tf32: bool) -> float:
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = tf32
    try:
        g = torch.Generator(device="cuda").manual_seed(1)
        a = torch.randn(n, n, device="cuda", dtype=dtype, generator=g)
        b = torch.randn(n, n, device="cuda", dtype=dtype, generator=g)
        c = torch.empty(n, n, device="cuda", dtype=dtype)
        for _ in range(2):
            torch.matmul(a, b, out=c)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        return 2.0 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def measure(quick: bool = False) -> dict:
    """TFLOP/s of cuBLAS FP32 (SIMT), TF32 and FP64 GEMMs on the current device."""
    n32, n64, reps = (4096, 2048, 3) if quick else (8192, 4096, 10)
    return {
        "fp32_simt_tflops": _gemm_tflops(torch.float32, n32, reps, tf32=False),
        "tf32_tflops": _gemm_tflops(torch.float32, n32, reps, tf32=True),
        "fp64_tflops": _gemm_tflops(torch.float64, n64, reps, tf32=False),
        "how": f"cuBLAS via torch.matmul, {n32}^3 (FP32, TF32) and {n64}^3 (FP64), 2 N^3 flops, best of {reps}, "
               "CUDA events",
        "device": torch.cuda.get_device_name(),
    }


if __name__ == "__main__":
    print(json.dumps(measure()))
