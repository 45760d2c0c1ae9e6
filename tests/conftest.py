import json
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def golden_problem(name, dim, rho=2400.0):
    from cudafemproject_gb300 import meshio
    return meshio.read_task(os.path.join(GOLDEN, "meshes", f"{dim}D", name), dim, E=2e7, nu=0.25, rho=rho)


def golden_ref(name):
    return np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))


def dyn_case(name):
    from cudafemproject_gb300 import meshio
    r = golden_ref(name)
    base = str(r["base"])
    dim = 2 if base.startswith("sq") else 3
    p = golden_problem(base, dim, rho=float(r["rho"]))
    wv = json.loads(str(r["wavelet"]))
    w = meshio.WaveletParams(wv["WaveletType"], float(np.float32(wv["freq"])), float(np.float32(wv["timeshift"])),
                             float(np.float32(wv["ampl"])))
    args = (float(np.float32(r["beta1"])), float(np.float32(r["beta2"])), float(np.float32(r["dt"])),
            float(np.float32(r["endtime"])))
    return p, w, args, r


STATIC_CASES = [("test_rect_pcg", 2), ("9task_3", 2), ("sq8", 2), ("sq16", 2), ("box3", 3), ("box4p", 3)]
SYNTH_CASES = [("sq8", 2), ("sq16", 2), ("box3", 3), ("box4p", 3)]
DYN_CASES = ["dyn_expl", "dyn_impl", "dyn_expl2d"]


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
