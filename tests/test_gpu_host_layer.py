"""The C++ mirror of the reference interface (dataKeeper, gpuCalculateFEM_EbE_vec,
gpuCalculateFEM_DYN, WriteResults) run from a run_config, through the C-ABI
entry cfem_run_task and through the cfem_run executable."""
import ctypes as C
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import GOLDEN, dyn_case, golden_problem, rel
from cudafemproject_gb300 import capi, meshio

pytestmark = pytest.mark.gpu


def _work(tmp_path, dim, tasks, extra=None):
    shutil.copytree(os.path.join(GOLDEN, "meshes", f"{dim}D"), tmp_path / "prepared_meshes" / f"{dim}D")
    (tmp_path / "fem_results" / f"{dim}D").mkdir(parents=True)
    for t in tasks:
        (tmp_path / "fem_results" / f"{dim}D" / t).mkdir()
    cfg = {"working_path": str(tmp_path) + "/", "task": tasks, "DIM": dim, "youngModulus": 2e7, "poissonRatio": 0.25}
    cfg.update(extra or {})
    path = tmp_path / "run_config.json"
    path.write_text(json.dumps(cfg))
    return str(path)


@pytest.mark.parametrize("name", ["test_rect_pcg", "9task_3"])
def test_run_task_static_golden(tmp_path, name):
    cfg = _work(tmp_path, 2, [name])
    p = golden_problem(name, 2)
    u = np.zeros(p.n_dof)
    info = capi.SolveInfo()
    st = capi.lib().cfem_run_task(cfg.encode(), name.encode(), 1, u.ctypes.data, u.size, C.byref(info), None)
    capi.check(st, "cfem_run_task")
    g = np.loadtxt(f"{GOLDEN}/{name}_vtk_displacements.txt")
    assert rel(u, g) < 2e-5  # default run_config: FP32, the reference's stopping rule
    vtk = tmp_path / "fem_results" / "2D" / name / "results.vtk"
    assert rel(meshio.read_vtk_displacements(str(vtk), 2), g) < 2e-5


def test_run_task_fp64_and_dynamic(tmp_path):
    cfg = _work(tmp_path, 3, ["box3"], {"gb300": {"precision": "fp64", "stop_rule": "residual", "tol": 1e-14}})
    p = golden_problem("box3", 3)
    u = np.zeros(p.n_dof)
    capi.check(capi.lib().cfem_run_task(cfg.encode(), b"box3", 0, u.ctypes.data, u.size, None, None), "run")
    x, _ = O.Oracle(p).static(tol=1e-14, rule=1)
    assert rel(u, x) <= 1e-10
    p, w, args, ref = dyn_case("dyn_expl")
    cfg = _work(tmp_path / "d", 3, ["box3"], {"task_type": "dynamic", "rho": 2000.0, "beta1": args[0], "beta2": args[1],
                                               "dt": args[2], "endtime": args[3],
                                               "wavelet": {"WaveletType": "ricker", "freq": 25.0, "ampl": 1.0},
                                               "gb300": {"precision": "fp64"}})
    u = np.zeros(p.n_dof)
    capi.check(capi.lib().cfem_run_task(cfg.encode(), b"box3", 0, u.ctypes.data, u.size, None, None), "run dyn")
    assert rel(u, ref["u"]) < 1e-4


def test_cfem_run_executable(tmp_path):
    from cudafemproject_gb300 import build
    cfg = _work(tmp_path, 2, ["test_rect_pcg", "9task_3"])
    r = subprocess.run([build.EXE, cfg], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    for name in ("test_rect_pcg", "9task_3"):
        vtk = tmp_path / "fem_results" / "2D" / name / "results.vtk"
        g = np.loadtxt(f"{GOLDEN}/{name}_vtk_displacements.txt")
        assert rel(meshio.read_vtk_displacements(str(vtk), 2), g) < 2e-5
    r = subprocess.run([build.EXE, str(tmp_path / "missing.json")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "cannot open" in r.stderr
