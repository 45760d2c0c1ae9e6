"""Seeded synthetic meshes in the reference's prepared-mesh form.

* :func:`square_2d`  unit square, n x n quads each cut into 2 CST triangles,
  left edge clamped (code 3), uniform traction on the right edge.
* :func:`box_3d`     lx x ly x lz box of nx x ny x nz hexes, each cut into 6
  Kuhn tetrahedra sharing the v000-v111 diagonal (conforming), interior nodes
  jittered by U(-j h, +j h) per axis, face z=0 clamped (code 7), a uniform
  traction on face z=lz and/or a point load.

Nodes are lexicographic (i fastest, then j, then k). Coordinates are rounded
to float32 so that the FP32 reference and the FP64 paths see the same
geometry. Tractions are written as ``stress.txt`` rows whose "normal" is the
traction direction and whose pressure is ``-|t|``, so that the reference's
face-load formula (-coeff * p * L * n, cpu_fem_utils.cpp:564-582) pushes along
the traction direction.
"""
from __future__ import annotations

import numpy as np

from .meshio import Problem

# Kuhn split of a hex with corners v0..v7 = (000,100,110,010,001,101,111,011) (dx,dy,dz)
_HEX_CORNERS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                         [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]], dtype=np.int64)
_KUHN = np.array([[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6],
                  [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]], dtype=np.int64)
_TET_FACES = np.array([[1, 2, 3, 0], [0, 2, 3, 1], [0, 1, 3, 2], [0, 1, 2, 3]])  # 3 face verts, opposite
_TRI_EDGES = np.array([[1, 2, 0], [0, 2, 1], [0, 1, 2]])


def _f32(a):
    return np.asarray(a, dtype=np.float64).astype(np.float32).astype(np.float64)


def square_2d(n: int = 64, E: float = 2e7, nu: float = 0.25, traction: float = 1e3) -> Problem:
    """Unit square, n x n quads x 2 CST (config: 8192 elements at n=64)."""
    xs = np.linspace(0.0, 1.0, n + 1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")        # node id = i + (n+1) j
    nodes = _f32(np.stack([X.ravel(), Y.ravel()], axis=1))
    nid = lambda i, j: i + (n + 1) * j
    I, J = np.meshgrid(np.arange(n), np.arange(n), indexing="xy")
    I, J = I.ravel(), J.ravel()
    v00, v10, v11, v01 = nid(I, J), nid(I + 1, J), nid(I + 1, J + 1), nid(I, J + 1)
    elems = np.empty((2 * n * n, 3), dtype=np.int32)
    elems[0::2] = np.stack([v00, v10, v11], axis=1)
    elems[1::2] = np.stack([v00, v11, v01], axis=1)
    left = np.where(np.isclose(nodes[:, 0], 0.0))[0]
    cons = np.stack([left, np.full_like(left, 3)], axis=1).astype(np.int32)
    fn, fe = _boundary_faces(elems, nodes[:, 0] >= 1.0 - 1e-12)
    F = len(fe)
    return Problem(dim=2, nodes=nodes, elems=elems, cons=cons,
                   load_node=np.zeros(0, np.int32), load_vec=np.zeros((0, 2)),
                   face_nodes=fn, face_elem=fe, face_normal=np.tile([1.0, 0.0], (F, 1)),
                   face_pressure=np.full(F, -abs(traction)), E=E, nu=nu)


def _boundary_faces(elems: np.ndarray, on_plane: np.ndarray):
    """Faces (edges in 2D) whose nodes all satisfy ``on_plane``; returns
    ([F, dim+1] face nodes + opposite node, [F] element ids) in element order."""
    nv = elems.shape[1]
    tab = _TRI_EDGES if nv == 3 else _TET_FACES
    rows, owners = [], []
    for f in range(tab.shape[0]):
        fv = elems[:, tab[f, :nv - 1]]
        hit = np.all(on_plane[fv], axis=1)
        idx = np.where(hit)[0]
        rows.append(np.concatenate([fv[idx], elems[idx, tab[f, nv - 1]][:, None]], axis=1))
        owners.append(idx)
    rows = np.concatenate(rows, axis=0)
    owners = np.concatenate(owners)
    order = np.argsort(owners, kind="stable")
    return rows[order].astype(np.int32), owners[order].astype(np.int32)


def box_3d(nx: int, ny: int, nz: int, lx: float = 1.0, ly: float = 1.0, lz: float = 4.0,
           jitter: float = 0.0, seed: int = 0, E: float = 2e7, nu: float = 0.25, rho: float = 2000.0,
           traction=(0.0, -1e3, 0.0), point_load=None, clamp_code: int = 7) -> Problem:
    """Kuhn-split tet box; face z=0 clamped, traction on z=lz, optional point load
    ``point_load=(node_id or 'top_centre', (fx, fy, fz))``."""
    h = np.array([lx / nx, ly / ny, lz / nz])
    gi, gj, gk = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    # lexicographic with i fastest: flatten in (k, j, i) order
    gi, gj, gk = (a.transpose(2, 1, 0).ravel() for a in (gi, gj, gk))
    nodes = np.stack([gi * h[0], gj * h[1], gk * h[2]], axis=1)
    if jitter > 0:
        rng = np.random.default_rng(seed)
        d = rng.uniform(-jitter, jitter, size=nodes.shape) * h
        interior = (gi > 0) & (gi < nx) & (gj > 0) & (gj < ny) & (gk > 0) & (gk < nz)
        nodes[interior] += d[interior]
    nodes = _f32(nodes)
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    HI, HJ, HK = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    HI, HJ, HK = (a.transpose(2, 1, 0).ravel() for a in (HI, HJ, HK))
    corner = np.stack([nid(HI + c[0], HJ + c[1], HK + c[2]) for c in _HEX_CORNERS], axis=1)
    elems = corner[:, _KUHN].reshape(-1, 4).astype(np.int32)
    base = np.where(gk == 0)[0]
    cons = np.stack([base, np.full_like(base, clamp_code)], axis=1).astype(np.int32)
    fn = np.zeros((0, 4), np.int32)
    fe = np.zeros(0, np.int32)
    normals = np.zeros((0, 3))
    press = np.zeros(0)
    t = np.asarray(traction, dtype=np.float64) if traction is not None else np.zeros(3)
    tmag = float(np.linalg.norm(t))
    if tmag > 0:
        fn, fe = _boundary_faces(elems, gk == nz)
        normals = np.tile(t / tmag, (len(fe), 1))
        press = np.full(len(fe), -tmag)
    load_node = np.zeros(0, np.int32)
    load_vec = np.zeros((0, 3))
    if point_load is not None:
        node, vec = point_load
        if node == "top_centre":
            node = nid(nx // 2, ny // 2, nz)
        load_node = np.array([node], np.int32)
        load_vec = _f32(np.asarray(vec, dtype=np.float64)[None, :])
    return Problem(dim=3, nodes=nodes, elems=elems, cons=cons, load_node=load_node, load_vec=load_vec,
                   face_nodes=fn, face_elem=fe, face_normal=normals, face_pressure=press,
                   E=E, nu=nu, rho=rho)


def random_tets(n_points: int = 800, seed: int = 7, E: float = 2e7, nu: float = 0.25, rho: float = 2000.0) -> Problem:
    """Unstructured tets: Delaunay tetrahedralisation (scipy) of uniform random
    points in the 1x1x4 box, slivers removed. Nodes with z < 0.3 are clamped (type 7); nodes
    with z > 3.7 carry a point load (0, -1e3, 0). Tet orientation as returned."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    nodes = rng.random((n_points, 3)) * np.array([1.0, 1.0, 4.0])
    elems = Delaunay(nodes).simplices.astype(np.int32)
    # drop slivers (quality 6 sqrt(2) V / l_max^3 below 0.1): they only add
    # rounding noise; the remaining mesh is still conforming (with voids)
    X = nodes[elems]
    vol = np.abs(np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]))) / 6
    edges = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    lmax = np.max([np.linalg.norm(X[:, a] - X[:, b], axis=1) for a, b in edges], axis=0)
    elems = elems[6 * np.sqrt(2) * vol / lmax ** 3 >= 0.1]
    used = np.zeros(n_points, bool)
    used[elems.ravel()] = True
    remap = np.cumsum(used) - 1
    nodes = nodes[used]
    elems = remap[elems].astype(np.int32)
    clamp = np.nonzero(nodes[:, 2] < 0.3)[0].astype(np.int32)
    cons = np.stack([clamp, np.full(len(clamp), 7, np.int32)], axis=1).astype(np.int32)
    top = np.nonzero(nodes[:, 2] > 3.7)[0].astype(np.int32)
    load_vec = np.tile(np.array([0.0, -1e3, 0.0]), (len(top), 1))
    return Problem(dim=3, nodes=nodes, elems=elems, cons=cons, load_node=top, load_vec=load_vec,
                   face_nodes=np.zeros((0, 4), np.int32), face_elem=np.zeros(0, np.int32),
                   face_normal=np.zeros((0, 3)), face_pressure=np.zeros(0), E=E, nu=nu, rho=rho)


def batch_boxes(n_boxes: int = 64, seed: int = 2, n_min: int = 8, n_max: int = 40, jitter: float = 0.2):
    """Independent tet boxes n x n x 4n (aspect 1:1:4, side counts uniform in
    [n_min, n_max]), each with E log-uniform in [1e6, 1e8] and nu uniform in
    [0.2, 0.4]; face z=0 clamped, traction 1e3 in -y on the top face; interior
    nodes jittered by +-jitter h (box i uses seed + 1 + i). Draw order: all
    side counts, then all E, then all nu."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(n_min, n_max + 1, size=n_boxes)
    Es = 10.0 ** rng.uniform(6, 8, size=n_boxes)
    nus = rng.uniform(0.2, 0.4, size=n_boxes)
    return [box_3d(int(n), int(n), 4 * int(n), jitter=jitter, seed=seed + 1 + i, E=float(E), nu=float(nu),
                   traction=(0.0, -1e3, 0.0)) for i, (n, E, nu) in enumerate(zip(ns, Es, nus))]


def cantilever_1p39m(seed: int = 0) -> Problem:
    """1x1x4 box, 48x48x192 hexes x 6 tets (2,654,208 tets, 1,390,179 DOF), jitter 0.2h."""
    return box_3d(48, 48, 192, jitter=0.2, seed=seed, traction=(0.0, -1e3, 0.0))


def elem_centroid_z(p: Problem) -> np.ndarray:
    return p.nodes[p.elems, 2].mean(axis=1)
