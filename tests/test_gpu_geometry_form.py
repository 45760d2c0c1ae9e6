"""The geometry edge-fan form (CFEM_FORM_GEOMETRY_FAN): the FP32 matvec forms
each tet's scaled gradients from streamed patch-relative FP32 coordinates.

Its FP32 products match the FP64 oracle to FP32 accuracy (the gradients
carry the rounding of the FP32 coordinate differences, about 1e-6 relative on
these meshes); FP64 solves and FP32 + FP64 refinement reach the same
tolerances as the stored-gradient forms; per-element moduli (set_young) and
the consistent-mass dynamics operator go through the same kernel.
"""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from cudafemproject_gb300 import meshgen
from cudafemproject_gb300.meshio import WaveletParams

pytestmark = pytest.mark.gpu


def _fp32_rel(ctx, o, x):
    x32 = x.astype(np.float32)
    return rel(ctx.matvec(x32, "fp32"), o.matvec(x32.astype(np.float64)))


@pytest.mark.parametrize("pe", [64, 768])
def test_matvec_jittered_box(pe):
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(14, 14, 48, jitter=0.2, seed=5, traction=(0.0, -1e3, 0.0))
    o = O.Oracle(p)
    ctx = FemContext(p, patch_elems=pe, matvec_form="geometry")
    assert ctx.counts()["matvec_form"] == 4
    rng = np.random.default_rng(4)
    for _ in range(2):
        x = rng.standard_normal(p.n_dof)
        assert rel(ctx.matvec(x, "fp64"), o.matvec(x)) < 1e-12
        assert _fp32_rel(ctx, o, x) < 2e-6


@pytest.mark.parametrize("pe", [96, 768])
def test_unstructured_tets(pe):
    """Delaunay tets: fans of every length, open and closed."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.random_tets(800, seed=7)
    o = O.Oracle(p, consistent=True)
    ctx = FemContext(p, semantics="consistent", patch_elems=pe, matvec_form="geometry")
    rng = np.random.default_rng(2)
    x = rng.standard_normal(p.n_dof)
    assert _fp32_rel(ctx, o, x) < 5e-6
    xo, _ = o.static(tol=1e-14, rule=1)
    u2, _ = ctx.static_solve("fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    assert rel(u2, xo) <= 1e-8


def test_refined_solve_matches_fp64():
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(6, 6, 24, jitter=0.2, seed=0, traction=(0.0, -1e3, 0.0))
    o = O.Oracle(p)
    xo, _ = o.static(tol=1e-14, rule=1)
    ctx = FemContext(p, matvec_form="geometry")
    u, info = ctx.static_solve("fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    assert rel(u, xo) <= 1e-8
    u64, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u64, xo) <= 1e-10


def test_set_young_scales():
    """Per-element moduli: the geometry blocks gain sqrt(E_e / E) rows."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(5, 5, 16, jitter=0.2, seed=3)
    rng = np.random.default_rng(9)
    y = p.E * np.exp(0.5 * rng.standard_normal(p.n_elems))
    ctx = FemContext(p, semantics="consistent", matvec_form="geometry")
    x = rng.standard_normal(p.n_dof)
    y0 = ctx.matvec(x.astype(np.float32), "fp32")
    ctx.set_young(y)
    q = meshgen.box_3d(5, 5, 16, jitter=0.2, seed=3)
    q.elem_E = y
    o = O.Oracle(q, consistent=True)
    assert _fp32_rel(ctx, o, x) < 2e-6
    assert rel(ctx.matvec(x.astype(np.float32), "fp32"), y0) > 1e-2
    xo, _ = o.static(tol=1e-14, rule=1)
    u, _ = ctx.static_solve("fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    assert rel(u, xo) <= 1e-8


@pytest.mark.parametrize("beta2", [0.0, 0.5])
def test_dynamics_fp32_matches_gradient_blocks(beta2):
    """FP32 GN22 steps (explicit lumped, implicit consistent mass): the
    geometry form follows the stored-gradient form to FP32 accuracy."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(3, 3, 8, jitter=0.15, seed=4, rho=2000.0, traction=None,
                       point_load=("top_centre", (0.0, 0.0, -1e3)))
    w = WaveletParams("ricker", 25.0, 0.0, 1.0)
    dt = 2e-5 if beta2 == 0 else 1e-3
    args = (0.5, beta2, dt, 40 * dt)
    kw = dict(precision="fp32", wavelet=w, pcg_tol=1e-7, stop_rule="residual")
    ug, _ = FemContext(p, semantics="consistent", matvec_form="geometry").dyn(*args, **kw)
    uf, _ = FemContext(p, semantics="consistent", matvec_form="fan").dyn(*args, **kw)
    o = O.Oracle(p, consistent=True)
    uo, _, _ = o.dyn(*args, wavelet=w, pcg_tol=1e-14, pcg_rule=1)
    assert rel(ug, uf) < 1e-4
    assert rel(ug, uo) < 1e-4
