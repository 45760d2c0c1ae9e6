"""Adjoint sensitivities and multi-RHS solves against the FP64 oracle."""
import numpy as np
import pytest

import oracle as O
from conftest import rel
from cudafemproject_gb300 import meshgen

pytestmark = pytest.mark.gpu


def _problem(seed=3):
    p = meshgen.box_3d(3, 3, 9, jitter=0.15, seed=seed, traction=(0.0, -1e3, 0.0))
    rng = np.random.default_rng(seed)
    p.elem_E = 2e7 * np.exp(0.5 * rng.standard_normal(p.n_elems))
    return p


def test_grad_young_vs_oracle_and_fd():
    from cudafemproject_gb300.solver import FemContext
    p = _problem()
    ctx = FemContext(p, semantics="consistent")
    o = O.Oracle(p, consistent=True)
    u, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    u = u.ravel()
    f = ctx.rhs()
    # compliance L = f.u  ->  dL/du = f
    dE, df, info = ctx.adjoint(u, f)
    lam, _ = o.pcg(f, tol=1e-14, rule=1)
    g_or = o.grad_E(lam, u)
    assert rel(dE, g_or) <= 1e-6
    assert rel(df, lam) <= 1e-9
    # central finite differences on a few elements (step 1e-4 relative)
    rng = np.random.default_rng(0)
    for e in rng.choice(p.n_elems, 5, replace=False):
        vals = []
        for s in (+1, -1):
            q = _problem()
            q.elem_E = q.elem_E.copy()
            q.elem_E[e] *= 1 + s * 1e-4
            c2 = FemContext(q, semantics="consistent")
            u2, _ = c2.static_solve("fp64", tol=1e-14, stop_rule="residual")
            vals.append(f @ u2.ravel())
        fd = (vals[0] - vals[1]) / (2e-4 * p.elem_E[e])
        assert abs(fd - dE[e]) <= 1e-4 * abs(dE[e]) + 1e-20, (e, fd, dE[e])


def test_set_young_matches_fresh_context():
    from cudafemproject_gb300.solver import FemContext
    p = _problem()
    ctx = FemContext(p, semantics="consistent")
    y2 = p.elem_E * 1.5
    ctx.set_young(y2)
    q = _problem()
    q.elem_E = y2
    u1, _ = ctx.static_solve("fp64", tol=1e-14, stop_rule="residual")
    u2, _ = FemContext(q, semantics="consistent").static_solve("fp64", tol=1e-14, stop_rule="residual")
    assert rel(u1, u2) < 1e-12


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32_refine", 1e-8)])
def test_multi_rhs(precision, tol):
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(3, 3, 9, jitter=0.2, seed=1)
    o = O.Oracle(p)
    rng = np.random.default_rng(7)
    F = rng.standard_normal((5, p.n_dof))
    ctx = FemContext(p)
    U, infos = ctx.pcg_multi(F, precision=precision, tol=1e-14 if precision == "fp64" else 1e-5,
                             stop_rule="residual", outer_tol=1e-13)
    for i in range(5):
        x, _ = o.pcg(F[i], tol=1e-14, rule=1)
        assert rel(U[i], x) <= tol


@pytest.mark.parametrize("form,pe", [("fan", 0), ("fan", 64), ("gradient", 0)])
def test_multi_rhs_batched(form, pe):
    """37 load cases (padded to 64) through the batched multi-RHS PCG, one of
    them zero, so whole passes of converged cases are skipped: every case
    matches the FP64 oracle and its own single-RHS solve. With 64 elements per
    patch the mesh has more patches than the grid has CTAs."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(10, 10, 40, jitter=0.2, seed=3)
    o = O.Oracle(p)
    rng = np.random.default_rng(11)
    F = rng.standard_normal((37, p.n_dof)) * 10.0 ** rng.uniform(2, 4, size=(37, 1))
    F[5] = 0.0
    ctx = FemContext(p, patch_elems=pe, matvec_form=form)
    U, infos = ctx.pcg_multi(F, precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    assert np.all(U[5] == 0.0)
    for i in (0, 1, 17, 36):
        x, _ = o.pcg(F[i], tol=1e-14, rule=1)
        assert rel(U[i], x) <= 1e-8, i
        assert infos[i]["status"] == 0 and infos[i]["rel_residual"] < 1e-11
    u_single, _ = ctx.pcg(F[17], "fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    assert rel(U[17], u_single) <= 1e-9
    U32, inf32 = ctx.pcg_multi(F[:9], precision="fp32", tol=1e-6, stop_rule="residual")
    for i in (0, 8):
        x, _ = o.pcg(F[i], tol=1e-14, rule=1)
        assert rel(U32[i], x) <= 1e-4, i


def test_torch_autograd_function():
    torch = pytest.importorskip("torch")
    from cudafemproject_gb300.autograd import static_solve
    from cudafemproject_gb300.solver import FemContext
    p = _problem(5)
    ctx = FemContext(p, semantics="consistent")
    young = torch.tensor(p.elem_E, dtype=torch.float64, requires_grad=True)
    f = torch.tensor(ctx.rhs(), dtype=torch.float64, requires_grad=True)
    u = static_solve(ctx, young, f, precision="fp64", tol=1e-13)
    loss = (f.detach() * u).sum() + 0.5 * (u[:30] ** 2).sum()
    loss.backward()
    o = O.Oracle(p, consistent=True)
    uo, _ = o.pcg(f.detach().numpy(), tol=1e-14, rule=1)
    g = f.detach().numpy().copy()
    g[:30] += uo[:30]
    lam, _ = o.pcg(g, tol=1e-14, rule=1)
    assert rel(young.grad.numpy(), o.grad_E(lam, uo)) <= 1e-6
    assert rel(f.grad.numpy(), lam) <= 1e-8


@pytest.mark.parametrize("side_stream", [False, True])
def test_torch_autograd_function_on_device(side_stream):
    """CUDA tensors in, CUDA tensors out: the forward solve and the adjoint read
    and write device memory only, on the caller's current torch stream (the
    default one, or a side stream whose inputs were produced there)."""
    torch = pytest.importorskip("torch")
    from cudafemproject_gb300.autograd import static_solve
    from cudafemproject_gb300.solver import FemContext
    p = _problem(5)
    ctx = FemContext(p, semantics="consistent")
    f_host = ctx.rhs()
    o = O.Oracle(p, consistent=True)
    uo, _ = o.pcg(f_host, tol=1e-14, rule=1)
    g = f_host.copy()
    g[:30] += uo[:30]
    lam, _ = o.pcg(g, tol=1e-14, rule=1)
    s = torch.cuda.Stream() if side_stream else torch.cuda.current_stream()
    with torch.cuda.stream(s):
        # inputs made on this stream (a scaled copy, so their producer is a kernel there)
        young = (torch.tensor(p.elem_E, dtype=torch.float64, device="cuda") * 1.0).requires_grad_(True)
        f = (torch.tensor(f_host, dtype=torch.float64, device="cuda") * 1.0).requires_grad_(True)
        u = static_solve(ctx, young, f, precision="fp64", tol=1e-13)
        assert u.is_cuda
        loss = (f.detach() * u).sum() + 0.5 * (u[:30] ** 2).sum()
        loss.backward()
    torch.cuda.synchronize()
    assert young.grad.is_cuda and f.grad.is_cuda
    assert rel(u.detach().cpu().numpy(), uo) <= 1e-10
    assert rel(young.grad.cpu().numpy(), o.grad_E(lam, uo)) <= 1e-6
    assert rel(f.grad.cpu().numpy(), lam) <= 1e-8


def _dyn_problem(E):
    p = meshgen.box_3d(2, 2, 5, jitter=0.1, seed=1, rho=2000.0, traction=None,
                       point_load=("top_centre", (0.0, 0.0, -1e3)))
    p.elem_E = E.copy()
    return p


def test_explicit_dynamics_adjoint_checkpointed():
    """Receiver-misfit gradient through 200 explicit steps (sqrt(N) = 15-step
    checkpoint segments) against the FP64 oracle's stored-state adjoint and
    central finite differences."""
    from cudafemproject_gb300.solver import FemContext
    rng = np.random.default_rng(3)
    p0 = _dyn_problem(np.full(120, 2e7))
    E = 2e7 * np.exp(0.3 * rng.standard_normal(p0.n_elems))
    p = _dyn_problem(E)
    top = np.where(np.isclose(p.nodes[:, 2], 4.0))[0].astype(np.int32)
    N, dt = 200, 1e-4
    T = float(np.float32(N * dt * 1.0000001))
    obs = 1e-7 * rng.standard_normal((N, len(top), 3))
    ctx = FemContext(p, semantics="consistent")
    L, g, info = ctx.dyn_adjoint(0.5, dt, T, top, obs)
    assert info["steps"] == N
    Lo, go = O.Oracle(p, consistent=True).dyn_adjoint(0.5, dt, T, top, obs)
    assert abs(L - Lo) <= 1e-10 * abs(Lo)
    assert rel(g, go) <= 1e-8
    big = np.argsort(-np.abs(g))[:4]
    for e in big:
        vals = []
        for s in (+1, -1):
            E2 = E.copy()
            E2[e] *= 1 + s * 1e-4
            Lq, _, _ = FemContext(_dyn_problem(E2), semantics="consistent").dyn_adjoint(0.5, dt, T, top, obs)
            vals.append(Lq)
        fd = (vals[0] - vals[1]) / (2e-4 * E[e])
        assert abs(fd - g[e]) <= 1e-4 * abs(g[e]), (e, fd, g[e])


def test_multi_rhs_many_cases():
    """130 load cases (padded to 256): the per-case grid sums take their
    thread-per-case form; cases still match the FP64 oracle."""
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(4, 4, 12, jitter=0.2, seed=6)
    o = O.Oracle(p)
    rng = np.random.default_rng(13)
    F = rng.standard_normal((130, p.n_dof)) * 10.0 ** rng.uniform(2, 4, size=(130, 1))
    ctx = FemContext(p)
    U, infos = ctx.pcg_multi(F, precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    for i in (0, 64, 129):
        x, _ = o.pcg(F[i], tol=1e-14, rule=1)
        assert rel(U[i], x) <= 1e-8, i
        assert infos[i]["status"] == 0


@pytest.mark.parametrize("cases_per_item", [2, 4, 8])
def test_multi_rhs_each_item_width(cases_per_item, monkeypatch):
    """The case-lane matvec at each chunk width (2, 4 or 8 cases per warp lane
    group, fixed through CFEM_MULTI_CASES): 11 cases (padded to 16) match the
    FP64 oracle, in FP32 + refinement and in plain FP32."""
    from cudafemproject_gb300.solver import FemContext
    monkeypatch.setenv("CFEM_MULTI_CASES", str(cases_per_item))
    p = meshgen.box_3d(6, 6, 20, jitter=0.2, seed=9)
    o = O.Oracle(p)
    rng = np.random.default_rng(17 + cases_per_item)
    F = rng.standard_normal((11, p.n_dof)) * 10.0 ** rng.uniform(2, 4, size=(11, 1))
    ctx = FemContext(p)
    U, infos = ctx.pcg_multi(F, precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-12)
    xs = {i: o.pcg(F[i], tol=1e-14, rule=1)[0] for i in (0, 5, 10)}
    for i, x in xs.items():
        assert rel(U[i], x) <= 1e-8, i
        assert infos[i]["status"] == 0
    U32, _ = ctx.pcg_multi(F, precision="fp32", tol=1e-6, stop_rule="residual")
    for i, x in xs.items():
        assert rel(U32[i], x) <= 1e-4, i


@pytest.mark.parametrize("cases_per_item", [2, 4, 8])
def test_multi_rhs_continued_refinement(cases_per_item, monkeypatch):
    """Multi-RHS FP32 + refinement with a loose inner tolerance (0.3): each
    case continues its last search direction across the FP64 true-residual
    replacements (stopped cases keep theirs), and every case still reaches the
    FP64 oracle's solution to 1e-8; one zero case stays zero."""
    from cudafemproject_gb300.solver import FemContext
    monkeypatch.setenv("CFEM_MULTI_CASES", str(cases_per_item))
    p = meshgen.box_3d(6, 6, 20, jitter=0.2, seed=12)
    o = O.Oracle(p)
    rng = np.random.default_rng(23)
    F = rng.standard_normal((13, p.n_dof)) * 10.0 ** rng.uniform(2, 4, size=(13, 1))
    F[4] = 0.0
    ctx = FemContext(p)
    U, infos = ctx.pcg_multi(F, precision="fp32_refine", tol=0.3, stop_rule="residual", outer_tol=1e-11,
                             max_outer=200)
    assert np.all(U[4] == 0.0)
    for i in (0, 7, 12):
        x, _ = o.pcg(F[i], tol=1e-14, rule=1)
        assert rel(U[i], x) <= 1e-8, i
        assert infos[i]["status"] == 0 and infos[i]["outer_iterations"] > 1
