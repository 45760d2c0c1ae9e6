"""LS-DYNA keyword reader (cudafemproject_gb300.kfile) on the CPU: the
reference's own raw meshes give the committed prepared meshes (made by the
reference's converter), and a written keyword file reads back."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from cudafemproject_gb300 import kfile, meshgen, meshio

# the reference checkout (moarseniy/CudaFEMproject), where one is present
REF_ROOT = os.environ.get("CFEM_REFERENCE_ROOT", "")
REF_RAW = os.path.join(REF_ROOT, "raw_meshes", "2D") if REF_ROOT else ""


@pytest.mark.parametrize("task", ["test_rect_pcg", "9task_3"])
def test_reference_raw_meshes_give_the_golden_prepared_meshes(task, tmp_path):
    if not REF_RAW:
        pytest.skip("CFEM_REFERENCE_ROOT (reference checkout) not set")
    raw = os.path.join(REF_RAW, task + ".k")
    if not os.path.exists(raw):
        pytest.skip("reference raw meshes not present")
    kfile.convert(raw, str(tmp_path / task), 2)
    a = meshio.read_task(str(tmp_path / task), 2)
    b = meshio.read_task(os.path.join(GOLDEN, "meshes", "2D", task), 2)
    for f in ("nodes", "elems", "cons", "load_node", "load_vec", "face_nodes", "face_elem", "face_normal",
              "face_pressure"):
        assert np.array_equal(getattr(a, f), getattr(b, f)), f


def test_keyword_round_trip_3d(tmp_path):
    p = meshgen.box_3d(3, 2, 5, jitter=0.2, seed=1, traction=(0.0, -1e3, 0.0))
    path = str(tmp_path / "box.k")
    kfile.write_k(p, path)
    q = kfile.read_k(path, 3)
    assert np.array_equal(q.nodes, p.nodes)
    assert np.array_equal(q.elems, p.elems)
    assert np.array_equal(np.sort(q.cons, axis=0), np.sort(p.cons, axis=0))
    assert np.array_equal(q.face_nodes[:, :3], p.face_nodes[:, :3])
    assert np.array_equal(q.face_elem, p.face_elem)
    assert np.array_equal(q.face_nodes[:, 3], p.face_nodes[:, 3])
    # normals: geometric, pointing away from the element's remaining node
    for fn, n in zip(q.face_nodes, q.face_normal):
        x = q.nodes[fn]
        assert np.dot(n, x[3] - x[0]) < 0
        assert np.allclose(np.cross(n, np.cross(x[1] - x[0], x[2] - x[0])), 0, atol=1e-12)


def test_spc_without_dofs_is_rejected(tmp_path):
    path = tmp_path / "bad.k"
    path.write_text("*NODE\n$\n1 0 0\n2 1 0\n3 0 1\n$\n*ELEMENT_SHELL\n1 1 1 2 3 3\n"
                    "*BOUNDARY_SPC_SET\n1 0 0 0 0\n*SET_NODE_LIST\n1\n1 2\n*END\n")
    with pytest.raises(ValueError):
        kfile.read_k(str(path), 2)


@pytest.mark.parametrize("dim", [2, 3])
def test_native_reader_matches_python_statement(tmp_path, dim):
    """The C++ reader (cfem_kfile_read) and the Python statement of the same
    rules give identical arrays, on written meshes and, when present, on the
    reference's raw meshes."""
    paths = []
    if dim == 3:
        p = meshgen.box_3d(4, 3, 6, jitter=0.2, seed=2, traction=(0.0, -1e3, 0.0))
    else:
        p = meshgen.square_2d(9, traction=1e3)
    path = str(tmp_path / f"m{dim}.k")
    kfile.write_k(p, path)
    paths.append(path)
    raw_dir = os.path.join(os.path.dirname(REF_RAW), f"{dim}D")
    if os.path.isdir(raw_dir):
        small = sorted((os.path.getsize(os.path.join(raw_dir, f)), f) for f in os.listdir(raw_dir) if f.endswith(".k"))
        paths += [os.path.join(raw_dir, f) for _, f in small[:4]]
    for path in paths:
        a = kfile.read_k(path, dim, native=True)
        b = kfile.read_k(path, dim, native=False)
        for f in ("nodes", "elems", "cons", "load_node", "load_vec", "face_nodes", "face_elem", "face_normal",
                  "face_pressure"):
            x, y = getattr(a, f), getattr(b, f)
            assert x.shape == y.shape and np.array_equal(x, y), (path, f)


def test_native_reader_rejects_bad_files(tmp_path):
    path = tmp_path / "bad.k"
    path.write_text("*NODE\n$\n1 0 0\n2 1 0\n$\n*ELEMENT_SHELL\n1 1 1 2 9 9\n*END\n")
    with pytest.raises(ValueError):
        kfile.read_k(str(path), 2)
    with pytest.raises(Exception):
        kfile.read_k(str(tmp_path / "missing.k"), 2)
