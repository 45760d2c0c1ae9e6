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


CALLER = r"""
// A caller written against the reference's interface (femfunc.h:20-24,
// fem_utils.h ElementsData), compiled against include/cfem_femfunc.hpp: the
// static flow of femfunc.cpp:3-23 with the reference's gpuPCG_EbE_vec
// argument list, then WriteResults(dk, ResultsDataKeeper&).
#include <cfem_femfunc.hpp>
#include <cstdio>
using namespace cfem_ref;
int main(int argc, char **argv) {
  dataKeeper dk(argv[1], argv[2]);
  ElementsData *ed = ElementsData::setElementsData(GB300, dk);
  ed->genMask();
  ed->calculateKlocals();
  ed->get_Klocals()->getDiagonal(6 * (dk.get_dim() - 1), *ed->get_diagK());
  ed->initFlocals(0.f, dk.getWaveletParams());
  ed->get_Flocals()->copy(*ed->get_r());
  gpuPCG_EbE_vec(*dk.get_displacements(), GB300, dk, *ed, true, 1e-8f, false);
  HostMatrix local;
  gpuPCG_EbE_vec(local, GB300, dk, *ed, false, 1e-8f, false);
  ResultsDataKeeper res(false, false, false, (int)dk.get_nodesCount());
  WriteResults(dk, res);
  FILE *f = std::fopen(argv[3], "wb");
  std::fwrite(dk.get_displacements()->get_data(), 4, dk.get_displacements()->get_numElements(), f);
  std::fwrite(local.get_data(), 4, local.get_numElements(), f);
  std::fwrite(ed->get_diagK()->get_data(), 4, ed->get_diagK()->get_numElements(), f);
  std::fclose(f);
  std::printf("%zu %zu %zu\n", dk.get_displacements()->get_numElements(), local.get_numElements(),
              ed->get_diagK()->get_numElements());
  delete ed;
  return 0;
}
"""


@pytest.mark.parametrize("name,dim", [("test_rect_pcg", 2), ("box3", 3)])
def test_reference_argument_lists_compile_and_solve(tmp_path, name, dim):
    """gpuPCG_EbE_vec(Matrix&, DEVICE_NAME, dataKeeper&, ElementsData&, bool,
    float, bool) and WriteResults(dataKeeper&, ResultsDataKeeper&) as the
    reference declares them, from a compiled C++ caller: the assembled result,
    the element-local result and the diagonal against the oracle."""
    import cudafemproject_gb300 as pkg
    pkg.lib()
    libdir = os.path.join(os.path.dirname(pkg.__file__), "_lib")
    inc = os.path.join(os.path.dirname(os.path.dirname(pkg.__file__)), "include")
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    exe = str(tmp_path / "caller")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", inc, str(src), "-o", exe, f"-L{libdir}", "-lcfem_gb300",
                    f"-Wl,-rpath,{libdir}"], check=True, capture_output=True)
    cfg = _work(tmp_path, dim, [name])
    out = tmp_path / "out.bin"
    r = subprocess.run([exe, cfg, name, str(out)], check=True, capture_output=True, text=True)
    n_u, n_loc, n_d = (int(v) for v in r.stdout.split())
    raw = np.fromfile(out, np.float32)
    p = golden_problem(name, dim)
    assert (n_u, n_loc, n_d) == (p.n_dof, p.n_elems * (dim + 1) * dim, p.n_dof)
    u, loc, diag = raw[:n_u], raw[n_u:n_u + n_loc], raw[n_u + n_loc:]
    o = O.Oracle(p)
    x, _ = o.static(tol=1e-14, rule=1)
    assert rel(u, x) < 1e-5  # FP32 PCG stopped by the reference's rule
    # a second solve of the same system, gathered per element (x_e = u[mask_e])
    assert rel(loc.reshape(p.n_elems, -1), u.reshape(-1, dim)[p.elems].reshape(p.n_elems, -1)) < 1e-6
    assert rel(diag, o.diag()) < 1e-6
    assert (tmp_path / "fem_results" / f"{dim}D" / name / "results.vtk").exists()
