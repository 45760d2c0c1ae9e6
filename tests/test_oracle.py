"""The oracle (oracle/fem_oracle.c) pinned against the reference's own outputs.

* FP32 element-local port == reference CPU build, bit for bit (fixtures made by
  tests/golden/make_golden.py from the unmodified reference sources);
* reference golden VTKs (testing/*_test/results.vtk);
* FP64 port == FP64 global form (same mathematics, different summation order).
"""
import numpy as np
import pytest

import oracle as O
from conftest import DYN_CASES, STATIC_CASES, SYNTH_CASES, dyn_case, golden_problem, golden_ref, rel, GOLDEN


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_port_f32_bit_exact_static(name, dim):
    p = golden_problem(name, dim)
    ref = golden_ref(f"static_{name}")
    u, it = O.ebe_static(p)
    assert it == int(ref["iterations"])
    assert np.array_equal(u, ref["u"])


@pytest.mark.parametrize("name,dim", SYNTH_CASES)
def test_port_f32_setup_arrays_bit_exact(name, dim):
    p = golden_problem(name, dim)
    ref = golden_ref(f"static_{name}")
    s = O.ebe_setup(p)
    assert np.array_equal(s["mask"], ref["mask"])
    assert np.array_equal(s["adj"], ref["adjElements"])
    assert np.array_equal(s["diagK"], ref["diagK"])
    assert np.array_equal(s["Flocals"], ref["Flocals"])
    assert np.array_equal(s["areas"], ref["areas"])
    if "Klocals" in ref.files:
        assert np.array_equal(s["Klocals"], ref["Klocals"])


@pytest.mark.parametrize("name", DYN_CASES)
def test_port_f32_bit_exact_dynamics(name):
    p, w, args, ref = dyn_case(name)
    u, steps, its = O.ebe_dyn(p, *args, wavelet=w)
    assert its == int(ref["pcg_iterations"])
    assert np.array_equal(u, ref["u"])


@pytest.mark.parametrize("name", ["test_rect_pcg", "9task_3"])
def test_golden_vtk(name):
    p = golden_problem(name, 2)
    g = np.loadtxt(f"{GOLDEN}/{name}_vtk_displacements.txt")
    u32, _ = O.ebe_static(p)
    assert rel(u32, g) < 3e-6  # the VTK holds 6 significant digits
    o = O.Oracle(p)
    x, _ = o.static(tol=1e-14, rule=1)
    assert rel(x, g) < 5e-6


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_port_f64_equals_global_form(name, dim):
    p = golden_problem(name, dim)
    u64, it = O.ebe_static(p, f64=True)
    o = O.Oracle(p)
    x, it2 = o.pcg(o.rhs(), tol=1e-8, rule=0)
    assert abs(it - it2) <= 1
    x2, _ = o.static(tol=1e-14, rule=1)
    assert rel(x2, O.ebe_static(p, eps=1e-30, f64=True)[0]) < 1e-9


@pytest.mark.parametrize("name", DYN_CASES)
def test_dyn_f64_port_equals_global_form(name):
    p, w, args, ref = dyn_case(name)
    u64, steps, its = O.ebe_dyn(p, *args, wavelet=w, f64=True)
    o = O.Oracle(p)
    ug, steps2, its2 = o.dyn(*args, wavelet=w)
    assert steps == steps2
    assert rel(ug, u64) < 5e-6  # implicit: both stop PCG at gamma < 1e-4 gamma0
    assert rel(ug, ref["u"]) < 1e-4


def test_oracle_bc_decode_q6():
    """Constraint codes UX=1, UY=2, UZ=3 decoded with &UX, &UY, &UZ (datakeeper.cpp:153-163)."""
    from cudafemproject_gb300 import meshgen
    p = meshgen.box_3d(1, 1, 1, traction=None)
    p.cons = np.array([[0, 1], [1, 2], [2, 3], [3, 4], [4, 5], [5, 6], [6, 7]], np.int32)
    b = O.Oracle(p).bc().reshape(-1, 3)
    expect = {1: [1, 0, 1], 2: [0, 1, 1], 3: [1, 1, 1], 4: [0, 0, 0], 5: [1, 0, 1], 6: [0, 1, 1], 7: [1, 1, 1]}
    for node, code in p.cons:
        assert b[node].tolist() == expect[int(code)], (node, code)


def test_consistent_traction_total_force():
    from cudafemproject_gb300 import meshgen
    p = meshgen.box_3d(3, 3, 6, traction=(0.0, -1e3, 0.0))
    f = O.Oracle(p, consistent=True).rhs().reshape(-1, 3)
    assert abs(f[:, 1].sum() - (-1e3 * 1.0 * 1.0)) < 1e-6
    assert abs(f[:, 0].sum()) < 1e-9


@pytest.mark.parametrize("name,dim", STATIC_CASES)
def test_assembled_form_equals_element_form(name, dim):
    """The node-block copy of K' (orc_assemble) multiplies like the element
    matrices and solves to the same answer, compat and consistent."""
    p = golden_problem(name, dim)
    for consistent in (False, True):
        o = O.Oracle(p, consistent=consistent)
        x = np.random.default_rng(3).standard_normal(o.ndof)
        y0 = o.matvec(x)
        f = o.rhs()
        u0, it0 = o.pcg(f, tol=1e-13, rule=1)
        o.assemble()
        assert rel(o.matvec(x), y0) < 1e-14
        u1, it1 = o.pcg(f, tol=1e-13, rule=1)
        assert rel(u1, u0) < 1e-11
        assert abs(it1 - it0) <= 2


def test_assembled_form_jittered_box_with_young_field():
    from cudafemproject_gb300 import meshgen
    p = meshgen.box_3d(4, 5, 12, jitter=0.2, seed=4)
    p.elem_E = 2e7 * np.exp(0.5 * np.random.default_rng(5).standard_normal(p.n_elems))
    o = O.Oracle(p, consistent=True)
    x = np.random.default_rng(6).standard_normal(o.ndof)
    y0 = o.matvec(x)
    o.assemble()
    assert rel(o.matvec(x), y0) < 1e-14


def test_warm_pcg_continues_to_tighter_tolerance():
    from cudafemproject_gb300 import meshgen
    p = meshgen.box_3d(4, 4, 16, jitter=0.2, seed=1)
    o = O.Oracle(p, consistent=True).assemble()
    f = o.rhs()
    xc, _ = o.pcg(f, tol=1e-13, rule=1)
    x6, _ = o.pcg(f, tol=1e-6, rule=1)
    xw, itw = o.pcg_warm(f, x6, tol=1e-13, rule=1)
    assert itw > 0
    assert rel(xw, xc) < 1e-11


def test_ebe_timer_runs_the_port_loop():
    from cudafemproject_gb300 import meshgen
    p = meshgen.box_3d(3, 3, 12)
    t = O.EbeTimer(p)
    assert t.setup_s >= 0 and t.init_s >= 0
    assert t.iters(3) >= 0
    t.close()
    assert O.num_threads() >= 1


@pytest.mark.parametrize("which", ["box", "square", "delaunay"])
def test_oracle_stress_of_an_affine_field(which):
    """strain = sym(grad u) exactly for u = A x on every element, whatever its
    orientation (the Delaunay tets come in both), and stress = D strain."""
    from cudafemproject_gb300 import meshgen
    p = {"box": lambda: meshgen.box_3d(3, 3, 6, jitter=0.2, seed=1), "square": lambda: meshgen.square_2d(6),
         "delaunay": lambda: meshgen.random_tets(300)}[which]()
    d = p.dim
    A = np.random.default_rng(0).standard_normal((d, d)) * 1e-3
    eps, sig, mis = O.Oracle(p).element_stress((p.nodes @ A.T).ravel())
    H = A
    if d == 3:
        exp = np.array([H[0, 0], H[1, 1], H[2, 2], H[0, 1] + H[1, 0], H[1, 2] + H[2, 1], H[0, 2] + H[2, 0]])
        lam = p.E * p.nu / ((1 + p.nu) * (1 - 2 * p.nu))
    else:
        exp = np.array([H[0, 0], H[1, 1], H[0, 1] + H[1, 0]])
        lam = p.E * p.nu / (1 - p.nu ** 2)  # plane stress
    mu = p.E / (2 * (1 + p.nu))
    assert np.abs(eps - exp).max() < 1e-11 * np.abs(exp).max()
    tr = exp[:d].sum()
    s_exp = np.concatenate([lam * tr + 2 * mu * exp[:d], mu * exp[d:]])
    assert np.abs(sig - s_exp).max() < 1e-9 * np.abs(s_exp).max()
