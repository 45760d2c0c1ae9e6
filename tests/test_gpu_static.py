"""GPU parity of the static path against the oracle and the reference fixtures.

Tolerances: FP64 paths <= 1e-10 relative to the converged FP64 oracle;
FP32 + FP64 refinement <= 1e-8; FP32-only results are held
to FP32 accuracy. DOF map, adjacency, constraint masks and renumbering are
bit-exact.
"""
import numpy as np
import pytest

import oracle as O
from conftest import STATIC_CASES, SYNTH_CASES, golden_problem, golden_ref, rel, GOLDEN
from cudafemproject_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctxs():
    from cudafemproject_gb300.solver import FemContext
    cache = {}

    def get(name, dim, semantics="compat", **kw):
        key = (name, dim, semantics, tuple(sorted(kw.items())))
        if key not in cache:
            cache[key] = (FemContext(golden_problem(name, dim), semantics=semantics, **kw), golden_problem(name, dim))
        return cache[key]
    return get


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_bit_exact_setup(ctxs, name, dim):
    ctx, p = ctxs(name, dim)
    o = O.Oracle(p)
    assert np.array_equal(ctx.dof_map(), o.mask())
    assert np.array_equal(ctx.adjacency(), o.adjacency())
    assert np.array_equal(ctx.bc_mask(), o.bc())
    n2o, e2o = ctx.renumbering()
    assert np.array_equal(np.sort(n2o), np.arange(p.n_nodes))
    assert np.array_equal(np.sort(e2o), np.arange(p.n_elems))
    ref = golden_ref(f"static_{name}")
    if "mask" in ref.files:
        assert np.array_equal(ctx.dof_map().astype(np.float32), ref["mask"])
        assert np.array_equal(ctx.adjacency().astype(np.float32), ref["adjElements"])


def test_renumbering_deterministic(ctxs):
    from cudafemproject_gb300.solver import FemContext
    p = golden_problem("box4p", 3)
    a = FemContext(p).renumbering()
    b = FemContext(p).renumbering()
    assert all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_element_matrices_and_diag(ctxs, name, dim):
    ctx, p = ctxs(name, dim)
    o = O.Oracle(p)
    k = ctx.element_matrices()
    ko = o.element_matrices()
    assert rel(k, ko) < 1e-12
    assert rel(ctx.diagonal(), o.diag()) < 1e-12
    ref = golden_ref(f"static_{name}")
    if "Klocals" in ref.files:  # the reference's FP32 Klocals (column-major per element)
        w = 6 * (dim - 1)
        kr = ref["Klocals"].reshape(-1, w, w).transpose(0, 2, 1)
        # the reference assembles K_e in FP32 from cofactor determinants
        assert rel(k, kr) < 2e-5
        assert rel(ko, kr) < 2e-5


@pytest.mark.parametrize("name,dim", STATIC_CASES)
@pytest.mark.parametrize("semantics", ["compat", "consistent"])
def test_rhs(ctxs, name, dim, semantics):
    ctx, p = ctxs(name, dim, semantics)
    o = O.Oracle(p, consistent=semantics == "consistent")
    assert rel(ctx.rhs(), o.rhs()) < 1e-13
    ref = golden_ref(f"static_{name}")
    if semantics == "compat" and "Flocals" in ref.files:
        # assembled reference Flocals
        fl = np.zeros(p.n_dof)
        np.add.at(fl, ref["mask"].astype(np.int64), ref["Flocals"].astype(np.float64))
        assert rel(ctx.rhs(), fl) < 1e-6


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_matvec(ctxs, name, dim):
    ctx, p = ctxs(name, dim)
    o = O.Oracle(p)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(p.n_dof)
    assert rel(ctx.matvec(x, "fp64"), o.matvec(x)) < 1e-13
    y32 = ctx.matvec(x.astype(np.float32), "fp32")
    assert rel(y32, o.matvec(x.astype(np.float32).astype(np.float64))) < 2e-6


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_static_fp64_reference_rule(ctxs, name, dim):
    """Same algorithm and stopping rule as gpuPCG_EbE_vec (eps 1e-8 on gamma):
    same iteration count as the FP64 oracle and the same iterate."""
    ctx, p = ctxs(name, dim)
    o = O.Oracle(p)
    xo, ito = o.pcg(o.rhs(), tol=1e-8, rule=0)
    u, info = ctx.static_solve("fp64", tol=1e-8, stop_rule="reference")
    # The iterates of a PCG stopped at this loose rule are rounding-sensitive:
    # two FP64 CPU implementations differing only in summation order already
    # differ by ~1e-6 at equal iteration counts. Parity <= 1e-10 is asserted on
    # converged solves (test_static_fp64_converged).
    assert abs(info["iterations"] - ito) <= 2
    assert rel(u, xo) < 1e-4
    ref = golden_ref(f"static_{name}")
    assert rel(u, ref["u"]) < 5e-4  # FP32 reference with the same loose stopping rule


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_static_fp64_converged(ctxs, name, dim):
    ctx, p = ctxs(name, dim)
    o = O.Oracle(p)
    xo, _ = o.static(tol=1e-14, rule=1)
    u, info = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u, xo) <= 1e-10
    assert info["rel_residual"] < 1e-11  # FP64 true-residual floor of the constrained operator


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_static_fp32_refine(ctxs, name, dim):
    ctx, p = ctxs(name, dim)
    o = O.Oracle(p)
    xo, _ = o.static(tol=1e-14, rule=1)
    u, info = ctx.static_solve("fp32_refine", tol=1e-5, stop_rule="residual", outer_tol=1e-12)
    assert rel(u, xo) <= 1e-8
    assert info["outer_iterations"] >= 1


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_static_fp32(ctxs, name, dim):
    ctx, p = ctxs(name, dim)
    o = O.Oracle(p)
    xo, _ = o.static(tol=1e-14, rule=1)
    u, info = ctx.static_solve("fp32", tol=1e-8, stop_rule="reference")
    assert rel(u, xo) < 1e-3


@pytest.mark.parametrize("name", ["test_rect_pcg", "9task_3"])
def test_golden_vtk_gpu(ctxs, name):
    ctx, p = ctxs(name, 2)
    g = np.loadtxt(f"{GOLDEN}/{name}_vtk_displacements.txt")
    u, _ = ctx.static_solve("fp32", tol=1e-8, stop_rule="reference")
    assert rel(u, g) < 2e-5
    u64, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u64, g) < 5e-6


def test_square_2d_64_fp64_vs_oracle():
    """The 64x64x2 CST configuration: FP64 Jacobi-PCG to relative residual 1e-12."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.square_2d(64)
    o = O.Oracle(p)
    xo, _ = o.static(tol=1e-14, rule=1)
    ctx = FemContext(p)
    u, info = ctx.static_solve("fp64", tol=1e-12, stop_rule="residual")
    assert info["rel_residual"] <= 1e-11  # FP64 true residual sits just above the recursive one
    assert rel(u, xo) <= 1e-9
    u2, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u2, xo) <= 1e-10


@pytest.mark.parametrize("form", ["gradient", "fan"])
def test_jittered_box_patch_sizes(form):
    """Results do not depend on the CTA patch size or on the element grouping
    (per element or per edge fan): locality layout only."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(6, 5, 14, jitter=0.2, seed=11)
    o = O.Oracle(p)
    xo, _ = o.static(tol=1e-14, rule=1)
    for pe in (64, 256, 1024):
        ctx = FemContext(p, patch_elems=pe, matvec_form=form)
        assert ctx.counts()["matvec_form"] == {"gradient": 1, "fan": 3}[form]
        u, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
        assert rel(u, xo) <= 1e-10, pe


@pytest.mark.parametrize("form", ["gradient", "fan"])
def test_many_patches_per_cta(form):
    """56k tets in patches of at most 64: every CTA walks several patches, so
    the double-buffered patch stream reuses each buffer several times."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(14, 14, 48, jitter=0.2, seed=5, traction=(0.0, -1e3, 0.0))
    o = O.Oracle(p)
    ctx = FemContext(p, patch_elems=64, matvec_form=form)
    assert ctx.counts()["n_patches"] > 3 * 152
    rng = np.random.default_rng(4)
    for _ in range(2):
        x = rng.standard_normal(p.n_dof)
        assert rel(ctx.matvec(x, "fp64"), o.matvec(x)) < 1e-12  # FP64 rounding, 56k tets
        y32 = ctx.matvec(x.astype(np.float32), "fp32")
        assert rel(y32, o.matvec(x.astype(np.float32).astype(np.float64))) < 2e-6


@pytest.mark.parametrize("form", ["gradient", "fan"])
@pytest.mark.parametrize("pe", [96, 768])
def test_unstructured_tets_both_forms(form, pe):
    """Delaunay mesh of random points: edge fans of every length 1..6, open and
    closed. Matvec and FP64 / refined solves against the oracle."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.random_tets(800, seed=7)
    o = O.Oracle(p, consistent=True)
    ctx = FemContext(p, semantics="consistent", patch_elems=pe, matvec_form=form)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(p.n_dof)
    assert rel(ctx.matvec(x, "fp64"), o.matvec(x)) < 1e-13
    y32 = ctx.matvec(x.astype(np.float32), "fp32")
    assert rel(y32, o.matvec(x.astype(np.float32).astype(np.float64))) < 2e-6
    xo, _ = o.static(tol=1e-14, rule=1)
    u, info = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u, xo) <= 1e-9
    u2, info2 = ctx.static_solve("fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    assert rel(u2, xo) <= 1e-8


def test_consistent_static(ctxs):
    ctx, p = ctxs("box4p", 3, "consistent")
    o = O.Oracle(p, consistent=True)
    xo, _ = o.static(tol=1e-14, rule=1)
    u, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u, xo) <= 1e-10


def test_pcg_explicit_rhs_and_torch_device_pointers(ctxs):
    torch = pytest.importorskip("torch")
    ctx, p = ctxs("box3", 3)
    o = O.Oracle(p)
    f = np.random.default_rng(5).standard_normal(p.n_dof)
    xo, _ = o.pcg(f, tol=1e-14, rule=1)
    u, info = ctx.pcg(f, "fp64", tol=1e-14, stop_rule="residual")
    assert rel(u, xo) <= 1e-10
    fd = torch.tensor(f, device="cuda")
    ud, _ = ctx.pcg(fd, "fp64", tol=1e-14, stop_rule="residual")
    assert rel(ud.cpu().numpy(), xo) <= 1e-10


def test_error_paths():
    from cudafemproject_gb300 import capi
    from cudafemproject_gb300.solver import FemContext
    p = golden_problem("sq8", 2)
    bad = golden_problem("sq8", 2)
    bad.nodes = np.vstack([bad.nodes, [[5.0, 5.0]]])  # unused node
    with pytest.raises(capi.CfemError) as e:
        FemContext(bad)
    assert e.value.status == capi.ERR_MESH
    flat = golden_problem("sq8", 2)
    flat.nodes = flat.nodes.copy()
    flat.nodes[:, 1] = 0.0  # zero-area elements
    with pytest.raises(capi.CfemError) as e:
        FemContext(flat)
    assert e.value.status == capi.ERR_MESH
    ctx = FemContext(p)
    f = np.full(p.n_dof, np.nan)
    with pytest.raises(capi.CfemError) as e:
        ctx.pcg(f, "fp64")
    assert e.value.status == capi.ERR_DIVERGED
    u, info = ctx.pcg(np.ones(p.n_dof), "fp64", tol=1e-30, stop_rule="residual", max_iter=3, allow_not_converged=True)
    assert info["status"] == capi.ERR_NOT_CONVERGED and info["iterations"] == 3
    # the context stays usable after the failures
    u, info = ctx.static_solve("fp64", tol=1e-12, stop_rule="residual")
    assert info["status"] == 0


@pytest.mark.parametrize("name", ["test_rect_pcg", "9task_3"])
def test_element_stress_golden(ctxs, name):
    """Element stresses / von Mises against the reference fixture's CELL_DATA."""
    import os
    path = f"{GOLDEN}/{name}_vtk_stress.txt"
    if not os.path.exists(path):
        pytest.skip("fixture without stress block")
    ctx, p = ctxs(name, 2)
    g = np.loadtxt(path)
    u, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    eps, sig, mis = ctx.element_stress(u)
    voigt = np.column_stack([g[:, 0], g[:, 4], g[:, 1]])  # xx, yy, xy
    assert rel(sig, voigt) < 2e-5
    assert rel(mis, g[:, 9]) < 2e-5


def test_autotune_patch_elems():
    """The autotuner returns one of its candidates, and a context built with it
    solves like the default one."""
    from cudafemproject_gb300.solver import FemContext, autotune_patch_elems
    p = meshgen.box_3d(8, 8, 24, jitter=0.2, seed=4)
    best, times = autotune_patch_elems(p, "consistent")
    assert best in times and all(t > 0 for t in times.values())
    ctx = FemContext(p, semantics="consistent", patch_elems="auto")
    assert ctx.patch_elems in times
    xo, _ = O.Oracle(p, consistent=True).static(tol=1e-14, rule=1)
    u, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u, xo) <= 1e-10



@pytest.mark.parametrize("loop", ["device", "host", "device_chunk6"])
@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_pcg_termination_3d(precision, loop, monkeypatch):
    """Stopping paths of the 3D PCG (bulk-copy FP32 fan matvec, FP64 fan
    matvec) whose scalars pass between the matvec and the update as block
    partials: a zero right-hand side stops before the first update; an
    iteration cap below, at and across the 16-iteration graph body stops at
    exactly that count, on the same iterate as the oracle's PCG after as many
    steps (so every alpha and beta of the recurrence agrees). Both loops: the
    graph WHILE node (default) and the host relaunching 16-iteration graphs
    (CFEM_HOST_LOOP, read when the context is created); and the WHILE node with
    6-iteration bodies (CFEM_PCG_CHUNK), so the caps fall inside, at the end of
    and past a body."""
    from cudafemproject_gb300 import capi
    from cudafemproject_gb300.solver import FemContext
    if loop == "host":
        monkeypatch.setenv("CFEM_HOST_LOOP", "1")
    else:
        monkeypatch.delenv("CFEM_HOST_LOOP", raising=False)
    if loop == "device_chunk6":
        monkeypatch.setenv("CFEM_PCG_CHUNK", "6")
    else:
        monkeypatch.delenv("CFEM_PCG_CHUNK", raising=False)
    p = meshgen.box_3d(4, 4, 12, jitter=0.2, seed=4)
    o = O.Oracle(p, consistent=True)
    ctx = FemContext(p, semantics="consistent")
    u, info = ctx.pcg(np.zeros(p.n_dof), precision, tol=1e-8, stop_rule="residual")
    assert info["status"] == 0 and info["iterations"] == 0 and np.all(u == 0.0)
    f = o.rhs()
    tol = 1e-10 if precision == "fp64" else 2e-4
    for m in (1, 2, 6, 12, 16, 17):
        u, info = ctx.pcg(f, precision, tol=1e-30, stop_rule="residual", max_iter=m, allow_not_converged=True)
        assert info["status"] == capi.ERR_NOT_CONVERGED and info["iterations"] == m, (m, info)
        x, its = o.pcg(f, tol=1e-30, rule=1, maxit=m, allow_maxit=True)
        assert its == m
        assert rel(u, x) <= tol, (m, rel(u, x))
    # and the same context still converges normally afterwards
    u, info = ctx.pcg(f, precision, tol=1e-11 if precision == "fp64" else 1e-5, stop_rule="residual")
    assert info["status"] == 0
    if precision == "fp64":
        x, _ = o.pcg(f, tol=1e-14, rule=1)
        assert rel(u, x) <= 1e-7


@pytest.mark.parametrize("name,dim", [("box3", 3), ("box4p", 3), ("sq8", 2)])
@pytest.mark.parametrize("consistent", [False, True])
def test_element_stress_vs_oracle(name, dim, consistent):
    """cfem_element_stress (strain, stress, von Mises per element) against the
    oracle's restatement of the reference's recovery (strain = B u_e, stress =
    D strain, deprecated/femfunc/femfunc.cpp:42-106) on the same displacement
    field: the oracle's FP64 static solution of the task, compat and
    consistent loads."""
    from cudafemproject_gb300.solver import FemContext
    p = golden_problem(name, dim)
    o = O.Oracle(p, consistent=consistent)
    u, _ = o.static(tol=1e-14, rule=1)
    ctx = FemContext(p, semantics="consistent" if consistent else "compat")
    eps, sig, mis = ctx.element_stress(u)
    e_o, s_o, m_o = o.element_stress(u)
    assert rel(eps, e_o) <= 1e-12
    assert rel(sig, s_o) <= 1e-12
    assert rel(mis, m_o) <= 1e-12


def test_element_stress_delaunay_with_young_field():
    """Unstructured tets of both orientations and per-element moduli."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.random_tets(400, seed=3)
    p.elem_E = 2e7 * np.exp(0.3 * np.random.default_rng(2).standard_normal(p.n_elems))
    o = O.Oracle(p, consistent=True)
    u = np.random.default_rng(5).standard_normal(p.n_dof) * 1e-3
    eps, sig, mis = FemContext(p, semantics="consistent").element_stress(u)
    e_o, s_o, m_o = o.element_stress(u)
    assert rel(eps, e_o) <= 1e-12
    assert rel(sig, s_o) <= 1e-12
    assert rel(mis, m_o) <= 1e-12


@pytest.mark.parametrize("inner", [0.2, 0.3, 0.5])
@pytest.mark.parametrize("mesh", ["box", "delaunay"])
def test_refinement_with_continued_directions(inner, mesh):
    """FP32 + FP64 refinement with a loose inner tolerance (a residual
    replacement factor from 0.2 up): the FP32 PCG keeps its search direction
    across the FP64 true-residual replacements and still reaches the oracle's
    solution to 1e-8."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(8, 8, 24, jitter=0.2, seed=5) if mesh == "box" else meshgen.random_tets(900, seed=4)
    ctx = FemContext(p, semantics="consistent")
    f = ctx.rhs()
    x, _ = O.Oracle(p, consistent=True).pcg(f, tol=1e-14, rule=1)
    u, info = ctx.pcg(f, "fp32_refine", tol=inner, stop_rule="residual", outer_tol=1e-10, max_outer=200)
    assert info["status"] == 0
    assert rel(u, x) <= 1e-8
    assert info["outer_iterations"] > 1


def test_copy_timeout_is_reported_and_context_recovers():
    """The failure path of the FP32 matvec's bulk copies, without a fault: a
    matvec whose first block of patch 0 is never requested, with the copy
    waits bounded at ~1 ms (cfem_selftest_copy_timeout). The kernel must give
    up, flag the missing copy and return, the host must report it, and the
    same context must then solve normally."""
    from cudafemproject_gb300 import capi
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(6, 6, 18, jitter=0.2, seed=2)
    ctx = FemContext(p, semantics="consistent")
    assert ctx.counts()["matvec_form"] == capi.FORM_GRADIENT_FAN
    L = capi.lib()
    for _ in range(2):
        assert L.cfem_selftest_copy_timeout(ctx._h) == capi.OK, L.cfem_last_error_string()
    f = ctx.rhs()
    x, _ = O.Oracle(p, consistent=True).pcg(f, tol=1e-14, rule=1)
    u, info = ctx.pcg(f, "fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    assert info["status"] == 0
    assert rel(u, x) <= 1e-8
    assert L.cfem_selftest_copy_timeout(FemContext(meshgen.square_2d(4))._h) == capi.ERR_UNSUPPORTED
