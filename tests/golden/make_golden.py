"""Regenerates the golden fixtures in tests/golden/ (run in a container that has
the reference checkout; the GPU tests only read the committed outputs).

    CFEM_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py [--ref <checkout>]

1. The reference's own LS-DYNA parser (mesh_parser_lib/fem_parser.py) turns
   raw_meshes/2D/{test_rect_pcg,9task_3}.k into prepared meshes (the committed
   testing/*_mesh/stress.txt is in an older 6-column format the current reader
   cannot parse). The displacement block of the reference's committed
   testing/<task>_test/results.vtk is stored beside them.
2. The reference's CPU path (oracle/_ref/ref_driver, built by oracle/ref.mk)
   is run on those meshes and on small seeded synthetic meshes; its float32
   outputs (static displacements, dynamics displacements and setup arrays)
   are stored as .npz.
3. A seeded receiver text file and node list are converted to SEG-Y by the
   reference's segyUtils convert() (``ref_driver segy``); the three files are
   stored under segy/ (``--only segy`` regenerates just these).
4. The reference's results writer (VTKfile.cpp MakeVTKfile2D/3D) writes the
   static solution of sq8 and box3 (``ref_driver vtk``, the same CPU solve as
   ref_static_<case>.npz); the files are stored under vtk/ (``--only vtk``).
"""
from __future__ import annotations

import argparse
import contextlib
import io
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from cudafemproject_gb300 import meshgen, meshio  # noqa: E402

DRIVER = os.path.join(REPO, "oracle", "_ref", "ref_driver")

# Synthetic cases, small enough for the reference's O(n_e * n_c) setup.
CASES = {
    "sq8": dict(kind="2d", n=8),
    "sq16": dict(kind="2d", n=16),
    "box3": dict(kind="3d", n=(3, 3, 12), jitter=0.2, seed=0),
    "box4p": dict(kind="3d", n=(4, 4, 8), jitter=0.15, seed=7, point=True),
}
DYN_CASES = {
    # explicit central difference (beta2 = 0), jittered so element masses differ
    "dyn_expl": dict(base="box3", rho=2000.0, beta1=0.5, beta2=0.0, dt=2e-5, endtime=2e-3,
                     wavelet=dict(WaveletType="ricker", freq=25.0, timeshift=0.0, ampl=1.0)),
    # implicit GN22 / Newmark (beta1 = 0.5, beta2 = 0.5)
    "dyn_impl": dict(base="box3", rho=2000.0, beta1=0.5, beta2=0.5, dt=1e-3, endtime=2e-2,
                     wavelet=dict(WaveletType="ricker", freq=25.0, timeshift=0.0, ampl=1.0)),
    # explicit, Berlage wavelet, 2D
    "dyn_expl2d": dict(base="sq8", rho=2000.0, beta1=0.5, beta2=0.0, dt=1e-5, endtime=1e-3,
                       wavelet=dict(WaveletType="berlage", freq=15.0, timeshift=0.0, ampl=1.0)),
}


def make_problem(spec):
    if spec["kind"] == "2d":
        return meshgen.square_2d(spec["n"], E=2e7, nu=0.25, traction=1e3)
    nx, ny, nz = spec["n"]
    pl = ("top_centre", (0.0, 0.0, -1e3)) if spec.get("point") else None
    return meshgen.box_3d(nx, ny, nz, jitter=spec["jitter"], seed=spec["seed"], E=2e7, nu=0.25,
                          traction=(0.0, -1e3, 0.0), point_load=pl)


def run_driver(mode, cfg_path, task, out):
    res = subprocess.run([DRIVER, mode, cfg_path, task, out], check=True, capture_output=True, text=True)
    return json.loads(res.stdout.strip().splitlines()[-1])


def write_cfg(work, dim, E, nu, extra=None):
    cfg = {"working_path": work, "DIM": dim, "youngModulus": E, "poissonRatio": nu}
    cfg.update(extra or {})
    path = os.path.join(work, "run_config.json")
    with open(path, "w") as f:
        json.dump(cfg, f)
    return path


def make_segy():
    """Receiver traces with zeros, negative zero and magnitudes 1e-12..1e5 at
    nodes with negative and almost-integer coordinates; 40 samples of 2.5 ms
    (interval above 32767 us, so the headers hold ms), velocity along y."""
    from cudafemproject_gb300 import segy
    dst = os.path.join(HERE, "segy")
    os.makedirs(dst, exist_ok=True)
    rng = np.random.default_rng(11)
    nodes = (rng.standard_normal((30, 2)) * 40).astype(np.float32)
    nodes[4] = [2.9999998, -0.75]
    with open(os.path.join(dst, "nodes.txt"), "w") as f:
        f.write(f"{len(nodes)}\n")
        for x in nodes:
            f.write(" ".join(repr(float(v)) for v in x) + "\n")
    times = np.arange(1, 41, dtype=np.float32) * np.float32(0.05)
    tr = (rng.standard_normal((40, 4)) * 10.0 ** rng.integers(-12, 6, (40, 4))).astype(np.float32)
    tr[0, 0] = 0.0
    tr[1, 1] = -0.0
    segy.write_receiver_text(os.path.join(dst, "receivers.txt"), [4, 17, 0, 29], times, tr)
    subprocess.run([DRIVER, "segy", os.path.join(dst, "reference.sgy"), os.path.join(dst, "receivers.txt"),
                    os.path.join(dst, "nodes.txt"), "2", "1", str(segy.VELOCITY), "123"], check=True,
                   capture_output=True)


def make_vtk():
    """The reference's results.vtk of the static sq8 and box3 solutions."""
    meshes = os.path.join(HERE, "meshes")
    os.makedirs(os.path.join(HERE, "vtk"), exist_ok=True)
    for name in ("sq8", "box3"):
        d = CASES[name]["kind"] == "2d" and 2 or 3
        p = make_problem(CASES[name])
        with tempfile.TemporaryDirectory() as work:
            shutil.copytree(os.path.join(meshes, f"{d}D"), os.path.join(work, "prepared_meshes", f"{d}D"))
            cfg = write_cfg(work, d, p.E, p.nu)
            run_driver("vtk", cfg, name, os.path.join(HERE, "vtk", f"{name}.vtk"))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CFEM_REFERENCE_ROOT"),
                    help="reference checkout (default: $CFEM_REFERENCE_ROOT)")
    ap.add_argument("--only", choices=["segy", "vtk"], default=None)
    args = ap.parse_args()
    if not args.ref:
        ap.error("the reference checkout is needed: --ref or CFEM_REFERENCE_ROOT")
    if not os.path.exists(DRIVER):
        subprocess.run(["make", "-f", "oracle/ref.mk", f"REF={args.ref}/FEMproject", "-j8"], cwd=REPO, check=True)
    if args.only == "vtk":
        make_vtk()
        return
    make_segy()
    if args.only == "segy":
        return
    sys.path.insert(0, args.ref)
    from mesh_parser_lib.fem_parser import run_parser  # the reference's own parser

    meshes = os.path.join(HERE, "meshes")
    # 1. reference fixtures
    for task in ("test_rect_pcg", "9task_3"):
        dst = os.path.join(meshes, "2D", task)
        os.makedirs(dst, exist_ok=True)
        with contextlib.redirect_stdout(io.StringIO()):
            run_parser(args.ref + "/", dst, os.path.join(args.ref, "raw_meshes", "2D", task + ".k"), task, 2)
        ref_vtk = os.path.join(args.ref, "testing", f"{task}_test", "results.vtk")
        u = meshio.read_vtk_displacements(ref_vtk, 2)
        np.savetxt(os.path.join(HERE, f"{task}_vtk_displacements.txt"), u, fmt="%.6g",
                   header=f"displacements block of testing/{task}_test/results.vtk (reference fixture)")
        lines = open(ref_vtk).read().split("\n")
        if "TENSORS stress double" in lines:
            i = lines.index("TENSORS stress double")
            rows = []
            j = i + 1
            while lines[j].strip():
                rows.append([float(v) for v in lines[j].split()])
                j += 1
            T = np.array(rows).reshape(-1, 9)
            k = lines.index("SCALARS mises_stress double")
            mises = np.array([float(v) for v in lines[k + 2:k + 2 + T.shape[0]]])
            np.savetxt(os.path.join(HERE, f"{task}_vtk_stress.txt"), np.column_stack([T, mises]), fmt="%.6g",
                       header=f"stress tensor (row-major 3x3) and mises_stress per cell of testing/{task}_test/results.vtk")
        with tempfile.TemporaryDirectory() as work:
            shutil.copytree(os.path.join(meshes, "2D"), os.path.join(work, "prepared_meshes", "2D"))
            cfg = write_cfg(work, 2, 2e7, 0.25)
            out = os.path.join(work, "u.bin")
            info = run_driver("static", cfg, task, out)
            uref = np.fromfile(out, dtype=np.float32).reshape(-1, 2)
            np.savez(os.path.join(HERE, f"ref_static_{task}.npz"), u=uref, iterations=info["pcg_iterations"])

    # 2. synthetic cases
    for name, spec in CASES.items():
        p = make_problem(spec)
        d = p.dim
        dst = os.path.join(meshes, f"{d}D", name)
        meshio.write_task(p, dst)
        with tempfile.TemporaryDirectory() as work:
            shutil.copytree(os.path.join(meshes, f"{d}D"), os.path.join(work, "prepared_meshes", f"{d}D"))
            cfg = write_cfg(work, d, p.E, p.nu)
            out = os.path.join(work, "u.bin")
            info = run_driver("static", cfg, name, out)
            u = np.fromfile(out, dtype=np.float32).reshape(-1, d)
            os.makedirs(os.path.join(work, "dump"))
            run_driver("dump", cfg, name, os.path.join(work, "dump"))
            rd = lambda f: np.fromfile(os.path.join(work, "dump", f), dtype=np.float32)
            extra = {}
            if p.n_elems <= 2000:
                extra["Klocals"] = rd("Klocals.bin")
            np.savez_compressed(os.path.join(HERE, f"ref_static_{name}.npz"), u=u, iterations=info["pcg_iterations"],
                                mask=rd("mask.bin"), adjElements=rd("adjElements.bin"), diagK=rd("diagK.bin"),
                                Flocals=rd("Flocals.bin"), areas=rd("elementsAreas.bin"),
                                constraintsIds=rd("constraintsIds.bin"), **extra)
    for name, spec in DYN_CASES.items():
        base = CASES[spec["base"]]
        p = make_problem(base)
        d = p.dim
        with tempfile.TemporaryDirectory() as work:
            shutil.copytree(os.path.join(meshes, f"{d}D"), os.path.join(work, "prepared_meshes", f"{d}D"))
            extra = dict(task_type="dynamic", rho=spec["rho"], beta1=spec["beta1"], beta2=spec["beta2"],
                         dt=spec["dt"], endtime=spec["endtime"], damping_alpha=0.0, damping_beta=0.0,
                         wavelet=spec["wavelet"])
            cfg = write_cfg(work, d, p.E, p.nu, extra)
            out = os.path.join(work, "u.bin")
            info = run_driver("dyn", cfg, spec["base"], out)
            u = np.fromfile(out, dtype=np.float32).reshape(-1, d)
            np.savez(os.path.join(HERE, f"ref_{name}.npz"), u=u, pcg_iterations=info["pcg_iterations"],
                     **{k: v for k, v in spec.items() if k not in ("base", "wavelet")},
                     base=spec["base"], wavelet=json.dumps(spec["wavelet"]))
    make_vtk()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
