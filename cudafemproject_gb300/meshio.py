"""Prepared-mesh text format and run_config JSON, as read by the reference.

The reference reads a task from ``<working_path>/prepared_meshes/<DIM>D/<task>/``
(FEMproject/DataKeeper/src/datakeeper.cpp:50-62, 116-213):

* ``nodes.txt``        N, then N rows of DIM coordinates
* ``elements.txt``     E, then E rows of DIM+1 zero-based node ids
* ``constraints.txt``  C, then C rows ``node type`` (Constraint::Type code,
  FEMproject/femstruct/src/femstruct.h:39-52)
* ``loads.txt``        L, then L rows ``node f_1 .. f_DIM``
* ``stress.txt``       F, then F rows ``DIM face nodes, opposite node,
  adjacent element, DIM normal components, pressure``

Every value is stored as ``float`` by the reference, so :func:`read_task`
rounds what it parses to float32 (``float32_inputs=True``); the same file then
gives bit-identical inputs here and in the reference. The run_config keys and
defaults follow datakeeper.cpp:6-48.
"""
from __future__ import annotations

import dataclasses
import json
import os
from typing import Optional

import numpy as np


@dataclasses.dataclass
class Problem:
    dim: int
    nodes: np.ndarray                 # [N, dim] float64
    elems: np.ndarray                 # [E, dim+1] int32
    cons: np.ndarray                  # [C, 2] int32 (node, type)
    load_node: np.ndarray             # [L] int32
    load_vec: np.ndarray              # [L, dim] float64
    face_nodes: np.ndarray            # [F, dim+1] int32 (face nodes + opposite node)
    face_elem: np.ndarray             # [F] int32
    face_normal: np.ndarray           # [F, dim] float64 (as written; normalised on use)
    face_pressure: np.ndarray         # [F] float64
    E: float = 2e7
    nu: float = 0.3
    rho: float = 2400.0
    elem_E: Optional[np.ndarray] = None  # [E] float64 per-element Young's modulus

    @property
    def n_nodes(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def n_elems(self) -> int:
        return int(self.elems.shape[0])

    @property
    def n_dof(self) -> int:
        return self.n_nodes * self.dim


@dataclasses.dataclass
class WaveletParams:
    """``wavelet`` block of run_config (datakeeper.cpp:37-47)."""
    wavelet_type: str = "default"     # "ricker", "berlage" or anything else (= no wavelet)
    freq: float = 15.0
    timeshift: float = 0.0
    ampl: float = 1.0

    @property
    def code(self) -> int:
        return {"ricker": 1, "berlage": 2}.get(self.wavelet_type, 0)


@dataclasses.dataclass
class RunConfig:
    """The reference's run_config keys with its defaults (datakeeper.cpp:6-48)."""
    dim: int
    task: list
    proj_dir: str = "undefined_path"
    work_dir: str = "undefined_path"
    young_modulus: float = 2e7
    poisson_ratio: float = 0.3
    save_segy: bool = False
    task_type: str = "static"
    rho: float = 2400.0
    beta1: float = 0.5
    beta2: float = 0.0
    damping_alpha: float = 0.0
    damping_beta: float = 0.0
    dt: float = 1e-3
    endtime: float = 0.1
    wavelet: WaveletParams = dataclasses.field(default_factory=WaveletParams)
    verbose: bool = True
    extra: dict = dataclasses.field(default_factory=dict)

    @property
    def is_dynamic(self) -> bool:
        # C++ compares "dynamic"; the Python driver upper-cases and compares
        # "DYNAMICS" (run_fem.py:21-23). Both spellings are accepted here.
        return self.task_type.lower() in ("dynamic", "dynamics")

    def prep_mesh_dir(self, task: str) -> str:
        return os.path.join(self.work_dir, "prepared_meshes", f"{self.dim}D", task)

    def res_dir(self, task: str) -> str:
        return os.path.join(self.work_dir, "fem_results", f"{self.dim}D", task)


def _f32(x):
    return np.asarray(x, dtype=np.float64).astype(np.float32).astype(np.float64)


def load_run_config(path: str) -> RunConfig:
    with open(path, "r") as f:
        cfg = json.load(f)
    if "DIM" not in cfg:
        raise KeyError("run_config: required key 'DIM' is missing")
    task = cfg.get("task", [])
    if isinstance(task, str):
        task = [task]
    rc = RunConfig(dim=int(cfg["DIM"]), task=list(task))
    rc.proj_dir = cfg.get("CudaFEMproject_path", rc.proj_dir)
    rc.work_dir = cfg.get("working_path", rc.work_dir)
    rc.young_modulus = float(np.float32(cfg.get("youngModulus", 2e7)))
    rc.poisson_ratio = float(np.float32(cfg.get("poissonRatio", 0.3)))
    rc.save_segy = bool(cfg.get("save_segy", False))
    rc.task_type = str(cfg.get("task_type", "static"))
    if rc.is_dynamic:
        rc.rho = float(np.float32(cfg.get("rho", 2400.0)))
        rc.beta1 = float(np.float32(cfg.get("beta1", 0.5)))
        rc.beta2 = float(np.float32(cfg.get("beta2", 0.0)))
        rc.damping_alpha = float(np.float32(cfg.get("damping_alpha", 0.0)))
        rc.damping_beta = float(np.float32(cfg.get("damping_beta", 0.0)))
        rc.dt = float(np.float32(cfg.get("dt", 1e-3)))
        rc.endtime = float(np.float32(cfg.get("endtime", 0.1)))
    if "wavelet" in cfg:
        w = cfg["wavelet"]
        rc.wavelet = WaveletParams(str(w.get("WaveletType", "default")), float(np.float32(w.get("freq", 15.0))),
                                   float(np.float32(w.get("timeshift", 0.0))), float(np.float32(w.get("ampl", 1.0))))
    rc.verbose = bool(cfg.get("verbose", True))
    rc.extra = {k: v for k, v in cfg.items() if k.startswith("gb300")}
    return rc


def _read_block(path: str, ncols: int, dtype=np.float64):
    with open(path, "r") as f:
        tokens = f.read().split()
    if not tokens:
        raise ValueError(f"{path}: empty file")
    n = int(float(tokens[0]))
    vals = tokens[1:1 + n * ncols]
    if len(vals) < n * ncols:
        raise ValueError(f"{path}: expected {n} rows of {ncols} values, got {len(vals)} values")
    arr = np.array([float(v) for v in vals], dtype=np.float64).reshape(n, ncols) if n else np.zeros((0, ncols))
    return arr.astype(dtype) if dtype is not np.float64 else arr


def read_task(mesh_dir: str, dim: int, E: float = 2e7, nu: float = 0.3, rho: float = 2400.0,
              float32_inputs: bool = True) -> Problem:
    """Read the five prepared-mesh files of one task (datakeeper.cpp:116-213)."""
    rnd = _f32 if float32_inputs else (lambda a: np.asarray(a, dtype=np.float64))
    nodes = rnd(_read_block(os.path.join(mesh_dir, "nodes.txt"), dim))
    elems = _read_block(os.path.join(mesh_dir, "elements.txt"), dim + 1).astype(np.int32)
    cons = _read_block(os.path.join(mesh_dir, "constraints.txt"), 2).astype(np.int32)
    loads = _read_block(os.path.join(mesh_dir, "loads.txt"), dim + 1)
    stress = _read_block(os.path.join(mesh_dir, "stress.txt"), (dim + 1) + 1 + dim + 1)
    return Problem(
        dim=dim, nodes=nodes, elems=elems, cons=cons,
        load_node=loads[:, 0].astype(np.int32), load_vec=rnd(loads[:, 1:]),
        face_nodes=stress[:, :dim + 1].astype(np.int32), face_elem=stress[:, dim + 1].astype(np.int32),
        face_normal=rnd(stress[:, dim + 2:2 * dim + 2]), face_pressure=rnd(stress[:, 2 * dim + 2]),
        E=float(np.float32(E)) if float32_inputs else E, nu=float(np.float32(nu)) if float32_inputs else nu,
        rho=float(np.float32(rho)) if float32_inputs else rho)


def _fmt(a) -> str:
    return " ".join(repr(float(v)) for v in a)


def write_task(p: Problem, mesh_dir: str) -> None:
    """Write the five prepared-mesh files; floats are written so that they parse back exactly."""
    os.makedirs(mesh_dir, exist_ok=True)

    def dump(name, n, rows):
        with open(os.path.join(mesh_dir, name), "w") as f:
            f.write(f"{n}\n")
            f.writelines(rows)

    fmt_f = "%.17g"
    with open(os.path.join(mesh_dir, "nodes.txt"), "w") as f:
        f.write(f"{p.n_nodes}\n")
        np.savetxt(f, p.nodes, fmt=fmt_f)
    with open(os.path.join(mesh_dir, "elements.txt"), "w") as f:
        f.write(f"{p.n_elems}\n")
        np.savetxt(f, p.elems, fmt="%d")
    dump("constraints.txt", len(p.cons), [f"{int(n)} {int(t)}\n" for n, t in p.cons])
    dump("loads.txt", len(p.load_node),
         [f"{int(n)} {_fmt(v)}\n" for n, v in zip(p.load_node, p.load_vec)])
    rows = []
    for i in range(len(p.face_elem)):
        rows.append(" ".join(str(int(v)) for v in p.face_nodes[i]) + f" {int(p.face_elem[i])} "
                    + _fmt(p.face_normal[i]) + f" {repr(float(p.face_pressure[i]))}\n")
    dump("stress.txt", len(p.face_elem), rows)


def write_run_config(path: str, rc: dict) -> None:
    with open(path, "w") as f:
        json.dump(rc, f, indent=1)


def read_vtk_displacements(path: str, dim: int) -> np.ndarray:
    """Displacement block of a legacy VTK written by the reference (VTKfile.cpp:281-386)."""
    out = []
    with open(path, "r") as f:
        lines = f.read().split("\n")
    for i, line in enumerate(lines):
        if line.startswith("VECTORS displacements"):
            j = i + 1
            while j < len(lines) and lines[j].strip():
                out.append([float(v) for v in lines[j].split()[:dim]])
                j += 1
            break
    return np.array(out, dtype=np.float64)
