"""Shared fixtures.  Tests marked ``gpu`` need a CUDA device; all others run on the CPU."""
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def lib():
    """libcalcir.so, built on first use (nvcc cross-compiles without a GPU)."""
    from calcir_gb300 import build
    build.build()
    import calcir_gb300
    return calcir_gb300


def load_golden(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        meta = json.load(f)
    data = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    return meta, data


def golden_params(meta):
    """Oracle parameter dictionary of a golden case (decoded like calcIR.cu:324-339)."""
    k = dict(meta["keys"])
    p = {"natom_mol": 4, "nchrom_mol": k.get("nchrom_mol", 2), "nzeros": k["nzeros"],
         "ntcfpoints": k["ntcfpoints"], "nsamples": k["nsamples"], "sampleEvery": k["sampleEvery"],
         "dt": k["dt"], "t1": k["t1"], "avef": k["avef"], "omegaStart": k["omegaStart"],
         "omegaStop": k["omegaStop"], "omegaStep": k["omegaStep"], "beginTime": k["beginTime"],
         "map": k["map"]}
    p["imodel"] = 1 if k["model"] in ("tip4p2005", "e3b3") else 0
    p["ispecies"] = {"H2O": 0, "HOD/D2O": 1, "HOD/H2O": 2, "D2O": 3}[k["species"]]
    return p


GOLDEN_CASES = ["small_h2o", "multi_d2o_map1", "hod_d2o", "bend_hod_h2o"]
