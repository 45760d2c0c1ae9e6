"""Host-side logic without a GPU: formats, config keys, mesh generator, ABI exports."""
import json
import os
import re

import numpy as np
import pytest

from conftest import REPO, golden_problem
from cudafemproject_gb300 import meshgen, meshio


def test_run_config_defaults(tmp_path):
    cfg = tmp_path / "c.json"
    cfg.write_text(json.dumps({"DIM": 3, "task": ["t"], "working_path": str(tmp_path)}))
    rc = meshio.load_run_config(str(cfg))
    assert rc.dim == 3 and rc.task == ["t"]
    assert rc.young_modulus == np.float32(2e7) and rc.poisson_ratio == np.float32(0.3)
    assert rc.task_type == "static" and not rc.is_dynamic
    assert rc.wavelet.code == 0
    cfg.write_text(json.dumps({"DIM": 2, "task_type": "dynamic", "beta2": 0.5, "wavelet": {"WaveletType": "ricker"}}))
    rc = meshio.load_run_config(str(cfg))
    assert rc.is_dynamic and rc.beta1 == 0.5 and rc.beta2 == 0.5 and rc.dt == np.float32(1e-3)
    assert rc.rho == np.float32(2400.0) and rc.wavelet.code == 1 and rc.wavelet.freq == 15.0
    cfg.write_text(json.dumps({"DIM": 2, "task_type": "DYNAMICS"}))
    assert meshio.load_run_config(str(cfg)).is_dynamic
    cfg.write_text(json.dumps({"task": []}))
    with pytest.raises(KeyError):
        meshio.load_run_config(str(cfg))


def test_prepared_mesh_roundtrip(tmp_path):
    p = meshgen.box_3d(3, 2, 4, jitter=0.2, seed=3, point_load=("top_centre", (0, 0, -5.0)))
    meshio.write_task(p, str(tmp_path))
    q = meshio.read_task(str(tmp_path), 3, E=p.E, nu=p.nu)
    for k in ("nodes", "elems", "cons", "load_node", "load_vec", "face_nodes", "face_elem", "face_normal", "face_pressure"):
        assert np.array_equal(getattr(p, k), getattr(q, k)), k


def test_meshgen_sizes():
    p = meshgen.square_2d(64)
    assert (p.n_elems, p.n_nodes, p.n_dof) == (8192, 4225, 8450)
    assert len(p.cons) == 65 and len(p.face_elem) == 64
    b = meshgen.box_3d(4, 4, 16)
    assert b.n_elems == 6 * 4 * 4 * 16 and b.n_nodes == 5 * 5 * 17
    # every tet positively or negatively oriented but never degenerate
    X = b.nodes[b.elems]
    v = np.linalg.det(X[:, 1:] - X[:, :1])
    assert np.all(np.abs(v) > 1e-12)
    # Kuhn split is conforming: every interior triangle is shared by exactly two tets
    faces = np.sort(np.concatenate([b.elems[:, [1, 2, 3]], b.elems[:, [0, 2, 3]], b.elems[:, [0, 1, 3]], b.elems[:, [0, 1, 2]]]), axis=1)
    _, cnt = np.unique(faces, axis=0, return_counts=True)
    assert cnt.max() == 2


def test_cantilever_counts_formula():
    nx, ny, nz = 48, 48, 192
    assert 6 * nx * ny * nz == 2654208
    assert (nx + 1) * (ny + 1) * (nz + 1) == 463393
    assert 3 * (nx + 1) * (ny + 1) * (nz + 1) == 1390179


def _declared_symbols():
    txt = open(os.path.join(REPO, "include", "cfem.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cfem_[a-z_0-9]+)\s*\(", txt)))


def test_abi_library_exports_declared_symbols():
    from cudafemproject_gb300 import build, capi
    build.build()
    import ctypes
    L = ctypes.CDLL(build.LIB)
    decl = _declared_symbols()
    assert len(decl) >= 20
    for s in decl:
        assert hasattr(L, s), s
    assert sorted(n for n, _, _ in capi.SIGNATURES) == decl
    assert L.cfem_abi_version() == 1


def test_abi_errors_without_gpu_work():
    """Invalid arguments are reported as status codes, never by exiting."""
    import ctypes as C
    from cudafemproject_gb300 import capi
    L = capi.lib()
    h = C.c_void_p()
    assert L.cfem_create(C.byref(h), None, None, None, None) == capi.ERR_INVALID_ARGUMENT
    assert b"null" in L.cfem_last_error_string()
    assert L.cfem_dof_map(None, None) == capi.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("name,dim", [("sq8", 2), ("box3", 3)])
def test_vtk_writer_byte_exact(tmp_path, name, dim):
    """results.vtk from cfem_write_vtk equals, byte for byte, the file the
    reference's own writer (VTKfile.cpp MakeVTKfile2D/3D) produced for the same
    mesh and the same FP32 displacements (the reference's CPU solve,
    tests/golden/ref_static_<case>.npz and tests/golden/vtk/<case>.vtk)."""
    import ctypes as C
    from cudafemproject_gb300 import capi
    from conftest import GOLDEN, golden_ref
    p = golden_problem(name, dim)
    u = np.ascontiguousarray(golden_ref(f"static_{name}")["u"], dtype=np.float32)
    nodes = np.ascontiguousarray(p.nodes, dtype=np.float64)
    elems = np.ascontiguousarray(p.elems, dtype=np.int32)
    assert u.shape == (p.n_nodes, dim)
    out = str(tmp_path / "results.vtk")
    st = capi.lib().cfem_write_vtk(out.encode(), dim, nodes.ctypes.data, p.n_nodes, elems.ctypes.data, p.n_elems,
                                   u.ctypes.data)
    assert st == capi.OK
    with open(out, "rb") as f, open(os.path.join(GOLDEN, "vtk", f"{name}.vtk"), "rb") as g:
        assert f.read() == g.read()
    assert capi.lib().cfem_write_vtk(out.encode(), 4, None, 0, None, 0, None) == capi.ERR_INVALID_ARGUMENT
