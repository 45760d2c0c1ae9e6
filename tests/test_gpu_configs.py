"""The batched, adjoint and dynamics configurations at mid sizes the FP64
oracle solves in seconds, each against the oracle (oracle/fem_oracle.c,
assembled node-block form on all host cores).

* 64 traction load cases on a 12x12x48 tet box as one multi-RHS PCG
  (FP32 + FP64 refinement): every case within 1e-8 of the oracle. Load cases
  are combinations of three unit tractions, so the oracle's solutions of those
  three give every case's reference answer by linearity.
* Adjoint gradient on a 16x16x64 tet cantilever with E_e = 2e7 exp(0.5 z_e):
  dL/dE and dL/df within 1e-6 of the oracle's (loss: compliance plus a sensor
  misfit against a second modulus field's displacements).
* Elastodynamics on a 16x16x128 tet column with a Ricker point force at the top
  centre (consistent semantics): 200 explicit steps and 20 implicit Newmark
  steps (beta 0.25, gamma 0.5), trajectories within 1e-9 of the oracle's.
"""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from cudafemproject_gb300 import meshgen
from cudafemproject_gb300.meshio import WaveletParams

pytestmark = pytest.mark.gpu


def test_multi_rhs_64_cases_box_12x12x48():
    from cudafemproject_gb300.solver import FemContext
    nx, ny, nz = 12, 12, 48
    basis = [meshgen.box_3d(nx, ny, nz, traction=t) for t in ((1.0, 0, 0), (0, 1.0, 0), (0, 0, 1.0))]
    E3 = np.stack([FemContext(b, semantics="consistent").rhs() for b in basis])
    p = meshgen.box_3d(nx, ny, nz)
    rng = np.random.default_rng(1)
    k = 64
    d = rng.standard_normal((k, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    C3 = d * (10.0 ** rng.uniform(2, 4, size=k))[:, None]
    F = C3 @ E3
    ctx = FemContext(p, semantics="consistent")
    U, infos = ctx.pcg_multi(F, precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-10)
    o = O.Oracle(p, consistent=True).assemble()
    assert np.allclose(E3, np.stack([O.Oracle(b, consistent=True).rhs() for b in basis]), rtol=0, atol=1e-12)
    X3 = np.stack([o.pcg(E3[i], tol=1e-13, rule=1)[0] for i in range(3)])
    Uo = C3 @ X3
    errs = [rel(U[i], Uo[i]) for i in range(k)]
    assert max(errs) <= 1e-8, max(errs)
    assert all(i["status"] == 0 for i in infos)


def test_adjoint_cantilever_16x16x64():
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(16, 16, 64, traction=(0.0, -1e3, 0.0))
    rng = np.random.default_rng(3)
    young = 2e7 * np.exp(0.5 * rng.standard_normal(p.n_elems))
    surf = np.nonzero((p.nodes[:, 0] <= 1e-9) | (p.nodes[:, 0] >= 1 - 1e-9) | (p.nodes[:, 1] <= 1e-9) |
                      (p.nodes[:, 1] >= 1 - 1e-9) | (p.nodes[:, 2] >= 4 - 1e-9))[0]
    sensors = rng.choice(surf, size=100, replace=False)
    young_obs = 2e7 * np.exp(0.5 * np.random.default_rng(4).standard_normal(p.n_elems))
    kw = dict(precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-13, max_iter=40000)
    p.elem_E = young_obs
    ctx = FemContext(p, semantics="consistent")
    f = ctx.rhs()
    o_obs = O.Oracle(p, consistent=True).assemble()
    u_obs = o_obs.pcg(f, tol=1e-13, rule=1)[0].reshape(-1, 3)[sensors]
    del o_obs
    p.elem_E = young
    ctx.set_young(young)
    u, _ = ctx.pcg(f, **kw)
    g = f.copy().reshape(-1, 3)
    g[sensors] += u.reshape(-1, 3)[sensors] - u_obs
    dE, df, _ = ctx.adjoint(u, g.ravel(), **kw)
    o = O.Oracle(p, consistent=True).assemble()
    uo, _ = o.pcg(f, tol=1e-13, rule=1)
    go = f.copy().reshape(-1, 3)
    go[sensors] += uo.reshape(-1, 3)[sensors] - u_obs
    lam, _ = o.pcg(go.ravel(), tol=1e-13, rule=1)
    assert rel(u, uo) <= 1e-9
    assert rel(dE, o.grad_E(lam, uo)) <= 1e-6
    assert rel(df, lam) <= 1e-6


@pytest.fixture(scope="module")
def column():
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(16, 16, 128, lz=8.0, E=2e7, nu=0.25, rho=2000.0, traction=(0.0, 0.0, 0.0),
                       point_load=("top_centre", (0.0, 0.0, -1.0)))
    return p, FemContext(p, semantics="consistent"), O.Oracle(p, consistent=True).assemble()


def test_explicit_200_steps_column_16x16x128(column):
    p, ctx, o = column
    w = WaveletParams("ricker", 25.0, 0.0, 1.0)
    dt = 5e-5  # below the stability limit of this mesh (about 3e-4)
    T = 200 * dt * 1.0000001
    ug, st, _ = o.dyn(0.5, 0.0, dt, T, wavelet=w)
    u, info = ctx.dyn(0.5, 0.0, dt, T, precision="fp64", wavelet=w)
    assert info["steps"] == st == 200
    assert np.linalg.norm(ug) > 0
    assert rel(u, ug) <= 1e-9


def test_implicit_newmark_20_steps_column_16x16x128(column):
    p, ctx, o = column
    w = WaveletParams("ricker", 25.0, 0.0, 1.0)
    dt = 1e-3
    T = 20 * dt * 1.0000001
    ug, st, _ = o.dyn(0.5, 0.5, dt, T, wavelet=w, pcg_tol=1e-14, pcg_rule=1)
    u, info = ctx.dyn(0.5, 0.5, dt, T, precision="fp64", wavelet=w, pcg_tol=1e-14, stop_rule="residual",
                      warm_start=True)
    assert info["steps"] == st == 20
    assert rel(u, ug) <= 1e-9
