"""LS-DYNA keyword (.k) meshes -> prepared meshes.

A restatement of how the reference's mesh converter
(mesh_parser_lib/parser_src/parser_lib.py:36-378, driven by
mesh_parser_lib/fem_parser.py) reads a keyword file, so that `.k` meshes made
for the reference load here unchanged:

* ``*NODE``: the line after the keyword is skipped (a column comment in the
  files the reference ships); then ``nid x y [z]`` lines up to a ``$`` line.
  Nodes keep file order; prepared ids are positions in that order.
* ``*ELEMENT_SOLID`` / ``*ELEMENT_SHELL``: ``eid pid n1 n2 ...`` lines up to
  the next keyword; the element's nodes are the first dim+1 after eid, pid.
* ``*SET_NODE_LIST``: the next line (stripped) is the set key; node ids follow.
* ``*BOUNDARY_SPC_SET``: ``sid cid dofx dofy [dofz]``; every node of set sid
  gets the constraint code of its flags (2D: x 1, y 2, xy 3; 3D: x 1, y 2,
  z 3, xy 4, xz 5, yz 6, xyz 7 -- the codes of femstruct.h:39-52).
* ``*DEFINE_CURVE``: the next line is the curve key; the value of a curve is
  the second number of its last data line.
* ``*LOAD_NODE_SET``: ``sid dof lcid``: every node of set sid gets the curve
  value along axis dof (1, 2, 3); with several cards the first matching one
  counts (what the reference's files end up holding).
* ``*LOAD_SEGMENT``: ``lcid sf at n1 n2 [n3 n4]``: the face n1 n2 (2D) or
  n1 n2 n3 (3D) of the first element (file order) that has all of them; the
  face row holds the face nodes, the element's remaining node, the element
  index, the face normal (2D (y2-y1, -(x2-x1)), 3D (p2-p1) x (p3-p1), not
  normalised, turned away from the remaining node) and the curve value as the
  pressure.

Where the reference would write a malformed file (an SPC set whose flags are
all zero, a load or segment naming a curve that does not exist) this reader
raises ``ValueError`` instead.

``read_k`` runs the library's C++ reader (csrc/kfile.cpp, the same rules; one
pass and hash maps, so multi-million-element meshes read in seconds); the
Python statement below it is kept as its readable counterpart and is compared
with it in the tests.
"""
from __future__ import annotations

import os
from typing import Dict, List

import numpy as np

from .meshio import Problem, write_task

_CODES2 = {(1, 0): 1, (0, 1): 2, (1, 1): 3}
_CODES3 = {(1, 0, 0): 1, (0, 1, 0): 2, (0, 0, 1): 3, (1, 1, 0): 4, (1, 0, 1): 5, (0, 1, 1): 6, (1, 1, 1): 7}


def _blocks(path: str):
    """(keyword, [lines]) in file order; lines keep their text (comments included)."""
    out = []
    cur = None
    with open(path) as f:
        for raw in f:
            line = raw.rstrip("\n")
            if line.startswith("*"):
                cur = (line.strip(), [])
                out.append(cur)
            elif cur is not None:
                cur[1].append(line)
    return out


def read_k(path: str, dim: int, E: float = 2e7, nu: float = 0.3, rho: float = 2400.0, native: bool = True) -> Problem:
    """Parse a keyword file into a Problem (prepared-mesh content, FP64 values).

    native: the library's C++ reader (cfem_kfile_read, linear in the file
    size); False runs the Python statement of the same rules below."""
    if native:
        return _read_k_native(path, dim, E, nu, rho)
    node_ids: List[str] = []
    coords: List[List[float]] = []
    elems_raw: List[List[str]] = []
    sets: Dict[str, List[str]] = {}
    spcs: List[List[str]] = []
    curves: Dict[str, str] = {}
    node_loads: List[List[str]] = []
    segments: List[List[str]] = []
    for kw, lines in _blocks(path):
        data = [ln for ln in lines if ln.strip() and not ln.lstrip().startswith("$")]
        if kw == "*NODE":
            for ln in lines[1:]:
                if ln.strip() == "$":
                    break
                if ln.lstrip().startswith("$") or not ln.strip():
                    continue
                tok = ln.split()
                node_ids.append(tok[0])
                coords.append([float(t) for t in tok[1:dim + 1]])
        elif kw in ("*ELEMENT_SOLID", "*ELEMENT_SHELL"):
            elems_raw.extend(ln.split()[2:2 + dim + 1] for ln in data)
        elif kw == "*SET_NODE_LIST" and data:
            key = data[0].strip()
            sets[key] = [t for ln in data[1:] for t in ln.split()]
        elif kw == "*BOUNDARY_SPC_SET" and data:
            spcs.append(data[0].split())
        elif kw == "*DEFINE_CURVE" and data:
            if len(data) > 1:
                curves[data[0].strip()] = data[-1].split()[1]
        elif kw == "*LOAD_NODE_SET" and data:
            node_loads.append(data[0].split())
        elif kw == "*LOAD_SEGMENT" and data:
            segments.append(data[0].split())
    index = {nid: i for i, nid in enumerate(node_ids)}
    nodes = np.array(coords, dtype=np.float64).reshape(-1, dim)
    elems = np.array([[index[t] for t in e] for e in elems_raw], dtype=np.int32).reshape(-1, dim + 1)

    # constraints
    cons = []
    codes = _CODES2 if dim == 2 else _CODES3
    for spc in spcs:
        flags = tuple(int(t) for t in spc[2:2 + dim])
        for key, members in sets.items():
            if spc[0] != key:
                continue
            if flags not in codes:
                raise ValueError(f"*BOUNDARY_SPC_SET {spc[0]}: no constrained DOF")
            cons.extend((index[m], codes[flags]) for m in members)
    cons_a = np.array(cons, dtype=np.int32).reshape(-1, 2)

    # nodal loads
    # several matching cards: the reference writes one block per card and its
    # mesh reader (datakeeper) takes the first block only
    matched = [ld for ld in node_loads if ld[0] in sets][:1]
    load_node, load_vec = [], []
    for ld in matched:
        if ld[2] not in curves:
            raise ValueError(f"*LOAD_NODE_SET names curve {ld[2]}, which is not defined")
        axis = int(ld[1]) - 1
        for m in sets[ld[0]]:
            v = [0.0] * dim
            v[axis] = float(curves[ld[2]])
            load_node.append(index[m])
            load_vec.append(v)

    # pressure faces
    face_to_elem = {}
    for ei, e in enumerate(elems):
        for skip in range(dim + 1):
            face = tuple(sorted(int(e[a]) for a in range(dim + 1) if a != skip))
            face_to_elem.setdefault(face, (ei, int(e[skip])))
    fnodes, felem, fnorm, fpress = [], [], [], []
    for seg in segments:
        if seg[0] not in curves:
            raise ValueError(f"*LOAD_SEGMENT names curve {seg[0]}, which is not defined")
        fn = [index[t] for t in seg[3:3 + dim]]
        hit = face_to_elem.get(tuple(sorted(fn)))
        if hit is None:
            raise ValueError(f"*LOAD_SEGMENT face {seg[3:3 + dim]} belongs to no element")
        ei, opp = hit
        x = nodes[fn]
        xb = nodes[opp]
        if dim == 2:
            n = np.array([x[1, 1] - x[0, 1], -(x[1, 0] - x[0, 0])])
        else:
            n = np.cross(x[1] - x[0], x[2] - x[0])
        if float(np.dot(n, xb - x[0])) > 0:
            n = -n
        fnodes.append(fn + [opp])
        felem.append(ei)
        fnorm.append(n)
        fpress.append(float(curves[seg[0]]))
    return Problem(dim=dim, nodes=nodes, elems=elems, cons=cons_a,
                   load_node=np.array(load_node, dtype=np.int32),
                   load_vec=np.array(load_vec, dtype=np.float64).reshape(-1, dim),
                   face_nodes=np.array(fnodes, dtype=np.int32).reshape(-1, dim + 1),
                   face_elem=np.array(felem, dtype=np.int32), face_normal=np.array(fnorm).reshape(-1, dim),
                   face_pressure=np.array(fpress, dtype=np.float64), E=E, nu=nu, rho=rho)


def _read_k_native(path: str, dim: int, E: float, nu: float, rho: float) -> Problem:
    import ctypes as C
    from . import capi
    L = capi.lib()
    h = C.c_void_p()
    st = L.cfem_kfile_read(os.fsencode(path), int(dim), C.byref(h))
    if st == capi.ERR_MESH:  # a malformed file: as the Python reader reports it
        raise ValueError(L.cfem_last_error_string().decode(errors="replace"))
    capi.check(st, "cfem_kfile_read")
    try:
        n = [C.c_int64() for _ in range(5)]
        capi.check(L.cfem_kfile_sizes(h, *[C.byref(v) for v in n]), "cfem_kfile_sizes")
        nn, ne, nc, nl, nf = (v.value for v in n)
        nodes = np.zeros((nn, dim), np.float64)
        elems = np.zeros((ne, dim + 1), np.int32)
        cons = np.zeros((nc, 2), np.int32)
        load_node = np.zeros(nl, np.int32)
        load_vec = np.zeros((nl, dim), np.float64)
        face_nodes = np.zeros((nf, dim + 1), np.int32)
        face_elem = np.zeros(nf, np.int32)
        face_normal = np.zeros((nf, dim), np.float64)
        face_pressure = np.zeros(nf, np.float64)
        arrs = (nodes, elems, cons, load_node, load_vec, face_nodes, face_elem, face_normal, face_pressure)
        capi.check(L.cfem_kfile_get(h, *[a.ctypes.data for a in arrs]), "cfem_kfile_get")
    finally:
        L.cfem_kfile_free(h)
    return Problem(dim=dim, nodes=nodes, elems=elems, cons=cons, load_node=load_node, load_vec=load_vec,
                   face_nodes=face_nodes, face_elem=face_elem, face_normal=face_normal,
                   face_pressure=face_pressure, E=E, nu=nu, rho=rho)


def convert(k_path: str, prepared_dir: str, dim: int) -> Problem:
    """The reference's run_parser step: keyword file -> the five prepared-mesh files."""
    p = read_k(k_path, dim)
    write_task(p, prepared_dir)
    return p


def write_k(p: Problem, path: str) -> None:
    """Keyword file of a Problem (nodes, elements, one constrained node set
    per constraint code, pressure faces with one curve each), in the subset
    that read_k understands. Node ids are 1-based positions."""
    dim = p.dim
    lines = ["*KEYWORD", "*NODE", "$    nid               x               y               z"]
    for i, x in enumerate(p.nodes):
        lines.append(f"{i + 1} " + " ".join(repr(float(v)) for v in x))
    lines.append("$")
    lines.append("*ELEMENT_SOLID" if dim == 3 else "*ELEMENT_SHELL")
    for i, e in enumerate(p.elems):
        lines.append(f"{i + 1} 1 " + " ".join(str(int(v) + 1) for v in e))
    codes = _CODES2 if dim == 2 else _CODES3
    flags_of = {c: f for f, c in codes.items()}
    sid = 0
    for code in sorted(set(int(c) for c in p.cons[:, 1])) if len(p.cons) else []:
        sid += 1
        members = [int(n) + 1 for n, c in p.cons if int(c) == code]
        lines += ["*BOUNDARY_SPC_SET", f"{sid} 0 " + " ".join(str(f) for f in flags_of[code]), "*SET_NODE_LIST",
                  f"{sid}"]
        lines += [" ".join(str(m) for m in members[k:k + 8]) for k in range(0, len(members), 8)]
    cid = 0
    for fn, pr in zip(p.face_nodes, p.face_pressure):
        cid += 1
        lines += ["*LOAD_SEGMENT", f"{cid} 1.0 0.0 " + " ".join(str(int(v) + 1) for v in fn[:dim]),
                  "*DEFINE_CURVE", f"{cid}", f"0.0 {repr(float(pr))}"]
    lines.append("*END")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
