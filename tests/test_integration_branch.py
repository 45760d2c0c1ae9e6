"""The GB300 branch for the reference's own femfunc library
(cudafemproject_gb300/integration/femfunc_gb300.cpp) compiled against the
reference's headers with oracle/ref.mk's include list and linked with the
reference's own objects and libcfem_gb300.so, on the CPU: the reference's
dataKeeper reads a prepared-mesh task, the branch widens it, and every array
(nodes, elements, constraint codes, point loads, boundary faces) must be the
task as the library's own prepared-mesh reader gives it, with constraint codes
that decode to the reference's DOF list. Needs CFEM_REFERENCE_ROOT (a
reference checkout); skipped without it."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, REPO

REF_ROOT = os.environ.get("CFEM_REFERENCE_ROOT", "")
pytestmark = pytest.mark.skipif(not REF_ROOT or not os.path.isdir(os.path.join(REF_ROOT, "FEMproject")),
                                reason="CFEM_REFERENCE_ROOT (reference checkout) not set")

MAIN = r"""
#include "femfunc_gb300.h"
#include <cstdio>
int main(int argc, char **argv) {
  dataKeeper dk(argv[1], argv[2]);
  const gb300::TaskArrays t = gb300::widen(dk);
  FILE *f = std::fopen(argv[3], "wb");
  auto wi = [&](const std::vector<int32_t> &v) { long long n = (long long)v.size(); std::fwrite(&n, 8, 1, f);
                                                  std::fwrite(v.data(), 4, v.size(), f); };
  auto wd = [&](const std::vector<double> &v) { long long n = (long long)v.size(); std::fwrite(&n, 8, 1, f);
                                                 std::fwrite(v.data(), 8, v.size(), f); };
  wd(t.nodes); wi(t.elems); wi(t.constraints); wi(t.load_nodes); wd(t.load_vectors);
  wi(t.face_nodes); wi(t.face_elems); wd(t.face_normals); wd(t.face_pressures);
  double mat[2] = {t.material.young_modulus, t.material.poisson_ratio};
  std::fwrite(mat, 8, 2, f);
  long long counts[5] = {t.mesh.n_nodes, t.mesh.n_elems, t.mesh.n_constraints, t.mesh.n_loads, t.mesh.n_faces};
  std::fwrite(counts, 8, 5, f);
  std::fclose(f);
  return 0;
}
"""


@pytest.fixture(scope="module")
def branch_exe(tmp_path_factory):
    ref = os.path.join(REF_ROOT, "FEMproject")
    mk = ["make", "-s", "-f", "oracle/ref.mk", f"REF={ref}"]
    subprocess.run(mk + ["-j8", "objs"], cwd=REPO, check=True)
    inc = subprocess.run(mk + ["print-inc"], cwd=REPO, check=True, capture_output=True, text=True).stdout.split()
    objs = subprocess.run(mk + ["print-objs"], cwd=REPO, check=True, capture_output=True, text=True).stdout.split()
    import cudafemproject_gb300 as pkg
    pkg.lib()  # builds libcfem_gb300.so
    libdir = os.path.join(REPO, "cudafemproject_gb300", "_lib")
    d = tmp_path_factory.mktemp("branch")
    main = d / "main.cpp"
    main.write_text(MAIN)
    exe = str(d / "branch")
    integ = os.path.join(REPO, "cudafemproject_gb300", "integration")
    cmd = (["g++", "-O1", "-std=c++17", "-w", "-I", integ, "-I", os.path.join(REPO, "include")] + inc +
           [str(main), os.path.join(integ, "femfunc_gb300.cpp"), "-o", exe, "-Wl,--start-group"] +
           [os.path.join(REPO, o) for o in objs] +
           ["-Wl,--end-group", f"-L{libdir}", "-lcfem_gb300", f"-Wl,-rpath,{libdir}"])
    subprocess.run(cmd, check=True, capture_output=True)
    return exe


def _read(path):
    out = []
    with open(path, "rb") as f:
        for dt in (np.float64, np.int32, np.int32, np.int32, np.float64, np.int32, np.int32, np.float64, np.float64):
            n = int(np.frombuffer(f.read(8), np.int64)[0])
            out.append(np.frombuffer(f.read(n * np.dtype(dt).itemsize), dt))
        mat = np.frombuffer(f.read(16), np.float64)
        counts = np.frombuffer(f.read(40), np.int64)
    return out, mat, counts


def _dofs(cons, dim):
    """DOFs constrained by (node, code) rows under the reference's decode
    (datakeeper.cpp:153-163: & UX, & UY, & UZ with UZ == 3)."""
    s = set()
    for node, code in cons.reshape(-1, 2):
        if code & 1:
            s.add(dim * node)
        if code & 2:
            s.add(dim * node + 1)
        if dim == 3 and code & 3:
            s.add(dim * node + 2)
    return s


@pytest.mark.parametrize("task,dim", [("test_rect_pcg", 2), ("9task_3", 2), ("sq8", 2), ("box3", 3), ("box4p", 3)])
def test_branch_widens_the_reference_task(branch_exe, tmp_path, task, dim):
    import json
    from cudafemproject_gb300 import meshio
    src = os.path.join(GOLDEN, "meshes", f"{dim}D", task)
    shutil.copytree(src, tmp_path / "prepared_meshes" / f"{dim}D" / task)
    cfg = tmp_path / "run_config.json"
    cfg.write_text(json.dumps({"working_path": str(tmp_path), "DIM": dim, "youngModulus": 2e7, "poissonRatio": 0.25}))
    out = tmp_path / "arrays.bin"
    subprocess.run([branch_exe, str(cfg), task, str(out)], check=True, capture_output=True)
    (nodes, elems, cons, lnodes, lvecs, fnodes, felems, fnorm, fpress), mat, counts = _read(out)
    p = meshio.read_task(src, dim, E=2e7, nu=0.25)
    f32 = lambda a: np.asarray(a, np.float64).astype(np.float32).astype(np.float64)
    assert np.array_equal(nodes, f32(p.nodes).ravel())
    assert np.array_equal(elems, p.elems.ravel())
    assert _dofs(cons, dim) == _dofs(p.cons.ravel(), dim)
    assert np.array_equal(lnodes, p.load_node.ravel())
    assert np.array_equal(lvecs, f32(p.load_vec).ravel())
    assert np.array_equal(fnodes, p.face_nodes.ravel())
    assert np.array_equal(felems, p.face_elem.ravel())
    n = p.face_normal.reshape(-1, dim)
    nrm = (n / np.linalg.norm(n, axis=1, keepdims=True)).ravel() if len(n) else n.ravel()
    assert np.allclose(fnorm, nrm, rtol=0, atol=1e-7)  # the reference normalises in float
    assert np.array_equal(fpress, f32(p.face_pressure).ravel())
    assert mat.tolist() == [2e7, float(np.float32(0.25))]
    assert counts.tolist() == [p.n_nodes, p.n_elems, len(cons) // 2, len(lnodes), len(felems)]
