"""ctypes binding of libcalcir.so (the C ABI declared in include/calcir.h).

Loading fails loudly when the library has not been built: there is no Python or CPU
implementation of the hot path behind this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcalcir.so")
EXE_PATH = os.path.join(HERE, "calcir")

CIR_OK = 0
ERRORS = {
    -1: "CIR_ERR_ARG", -2: "CIR_ERR_CUDA", -3: "CIR_ERR_NOMEM", -4: "CIR_ERR_NOCONVERGE",
    -5: "CIR_ERR_IO", -6: "CIR_ERR_PARSE", -7: "CIR_ERR_STATE", -8: "CIR_ERR_NONFINITE",
    -9: "CIR_ERR_NODEVICE",
}
PREC = {"fp32": 0, "tf32": 1, "bf16x3": 2}
STRLEN = 256


class CirError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [
        ("xtcf", C.c_char * STRLEN), ("outf", C.c_char * STRLEN), ("cptf", C.c_char * STRLEN),
        ("model", C.c_char * STRLEN), ("species", C.c_char * STRLEN),
        ("ntcfpoints", C.c_int), ("nsamples", C.c_int), ("sampleEvery", C.c_float),
        ("omegaStep", C.c_int), ("natom_mol", C.c_int), ("nchrom_mol", C.c_int), ("nzeros", C.c_int),
        ("map", C.c_int), ("dt", C.c_float), ("t1", C.c_float), ("avef", C.c_float),
        ("beginTime", C.c_float), ("omegaStart", C.c_float), ("omegaStop", C.c_float),
        ("imodel", C.c_int), ("ispecies", C.c_int),
        ("synth_nmol", C.c_int), ("synth_seed", C.c_int), ("synth_frame_dt", C.c_float),
        ("synth_sigma_trans", C.c_float), ("synth_sigma_rot", C.c_float),
        ("precision", C.c_int), ("batch_frames", C.c_int), ("verbose", C.c_int),
        ("cuda_graphs", C.c_int), ("autotune", C.c_int),
        ("propagate_vectors", C.c_int), ("share_frames", C.c_int), ("refine_eigen", C.c_int),
        ("test_stall_gemm", C.c_int), ("test_sweep_cap", C.c_int),
    ]


class Result(C.Structure):
    _fields_ = [
        ("tcf_ir", C.POINTER(C.c_double)), ("tcf_vv", C.POINTER(C.c_double)), ("tcf_vh", C.POINTER(C.c_double)),
        ("omega", C.POINTER(C.c_float)), ("sw", C.POINTER(C.c_float)), ("pw", C.POINTER(C.c_float)),
        ("rw", C.POINTER(C.c_float)), ("rmw", C.POINTER(C.c_float)),
        ("ls_omega", C.POINTER(C.c_float)), ("ls_ir", C.POINTER(C.c_float)), ("ls_vv", C.POINTER(C.c_float)),
        ("ls_vh", C.POINTER(C.c_float)), ("nls", C.c_int), ("bins_out_of_range", C.c_longlong),
        ("frame_steps_per_s", C.c_double),
    ]


class TrajIn(C.Structure):
    _fields_ = [
        ("natoms", C.c_int), ("nframes", C.c_int), ("xyz", C.c_void_p), ("box", C.c_void_p),
        ("frame_of_step", C.c_void_p),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("kernel_launches", C.c_longlong), ("eig_sweeps", C.c_longlong), ("frame_steps", C.c_longlong),
        ("ms_build", C.c_double), ("ms_eig", C.c_double), ("ms_prop", C.c_double), ("ms_tcf", C.c_double),
        ("ms_tridiag", C.c_double), ("eig_matrices", C.c_longlong),
        ("tuned_split_tile", C.c_int), ("tuned_tridiag_blocks", C.c_int),
    ]


class Synth(C.Structure):
    _fields_ = [
        ("nmol", C.c_int), ("seed", C.c_uint64), ("box_nm", C.c_double), ("frame_dt", C.c_double),
        ("sigma_trans", C.c_double), ("sigma_rot_deg", C.c_double), ("jitter", C.c_double),
        ("min_contact", C.c_double), ("max_tries", C.c_int),
    ]


# (name, argtypes) of every exported entry point; restype is int unless listed in _RESTYPE
P = C.c_void_p
SIGNATURES = {
    "cir_version": [], "cir_last_error": [],
    "cir_params_default": [C.POINTER(Params)],
    "cir_params_parse_file": [C.c_char_p, C.POINTER(Params)],
    "cir_params_finalize": [C.POINTER(Params)],
    "cir_nomega": [C.POINTER(Params)],
    "cir_result_sizes": [C.POINTER(Params), C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)],
    "cir_frame_index": [C.POINTER(Params), C.c_float, C.c_int, C.c_int, C.POINTER(C.c_int)],
    "cir_write_outputs": [C.POINTER(Params), C.POINTER(Result)],
    "cir_synth_default": [C.POINTER(Synth), C.c_int],
    "cir_synth_trajectory": [C.POINTER(Synth), C.c_int, P, P, C.POINTER(C.c_longlong)],
    "cir_traj_write": [C.c_char_p, C.c_int, C.c_int, C.c_float, P, P, P],
    "cir_traj_info": [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_float)],
    "cir_traj_read": [C.c_char_p, C.c_int, C.c_int, P, P, P],
    "cir_create": [C.POINTER(Params), C.c_int, C.POINTER(P)],
    "cir_destroy": [P],
    "cir_set_stream": [P, P],
    "cir_synchronize": [P],
    "cir_get_stats": [P, C.POINTER(Stats)],
    "cir_reset_stats": [P],
    "cir_build_hamiltonian": [P, C.c_int, P, P, P, P, P, P],
    "cir_eigh": [P, C.c_int, C.c_int, P, P],
    "cir_eigh_noalloc": [C.c_int, C.c_int, P, P, P],
    "cir_tridiag_sbr": [P, C.c_int, C.c_int, P, P, P, P],
    "cir_propagate": [P, C.c_int, C.c_int, P, P, C.c_float, P],
    "cir_tcf_terms": [P, C.c_int, P, P, P, P, P, P],
    "cir_spectral_density": [P, C.c_int, P, P, P, P],
    "cir_lineshape": [P, P, P, P, C.POINTER(C.c_int)],
    "cir_run": [P, C.c_int, P, P, P, C.POINTER(Result)],
    "cir_run_multi": [P, C.c_int, C.POINTER(TrajIn), C.POINTER(Result)],
    "cir_xtc_write": [C.c_char_p, C.c_int, C.c_int, P, P, P, C.c_float],
    "cir_get_coeffs": [P, P],
    "cir_set_coeffs": [P, P],
    "cir_loss_grad": [P, C.c_int, P, P, P, P, P, C.c_int, P, P],
}
_RESTYPE = {"cir_version": C.c_char_p, "cir_last_error": C.c_char_p}

_lib = None


def load() -> C.CDLL:
    """Load libcalcir.so (built by calcir_gb300.build); raises if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run calcir_gb300.build.build() first")
        lib = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPE.get(name, C.c_int)
        _lib = lib
    return _lib


def check(rc: int) -> None:
    if rc != CIR_OK:
        raise CirError(rc, load().cir_last_error().decode(errors="replace"))


def ptr(a) -> C.c_void_p | None:
    """Address of a numpy array, an int device address, or None."""
    if a is None:
        return None
    if isinstance(a, int):
        return C.c_void_p(a)
    if isinstance(a, np.ndarray):
        assert a.flags["C_CONTIGUOUS"], "arrays passed to the C ABI must be C-contiguous"
        return C.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    raise TypeError(f"cannot pass {type(a)} to the C ABI")
