"""Pins the CPU restatement (oracle/) to the reference's own outputs.

The golden fixtures hold what the reference code itself computed on each case
(tests/golden/make_golden.py).  The oracle runs the same inputs (same node and
element numbering) and must reproduce: basis tables and quadrature data,
neighbour lists bit-exact (order included), the matrix patterns bit-exact,
matrix values and right-hand sides within 1e-12 relative, and the solution
within 1e-10 relative L2.  The ILLT factor itself is a restatement of Eigen's
IncompleteCholesky (Eigen is absent), so only the converged solution pins it.
"""
import numpy as np
import pytest

import golden_cases as gc


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="module", params=gc.STATIONARY_2D)
def solved(request, oracle_lib):
    fx = gc.load(request.param)
    prob = gc.oracle_problem(fx)
    prob.find_neighbours(fx["config"].get("strategy", "MAX"))
    prob.assemble()
    prob.assemble_local()
    prob.solve(variant=0, tol=1e-14, maxit=20000, true_residual=True)
    return request.param, fx, prob


def test_basis_tables(solved):
    _, fx, prob = solved
    for name in ["basis_qN", "basis_qNxi", "basis_qNeta", "basis_weights", "basis_centre"]:
        np.testing.assert_allclose(prob.get(name), fx[name].reshape(-1), rtol=0, atol=2e-15, err_msg=name)


def test_quadrature_data(solved):
    _, fx, prob = solved
    for name in ["qcoords", "jacobians", "derivatives", "centres"]:
        ref = fx[name].reshape(-1)
        np.testing.assert_allclose(prob.get(name), ref, rtol=1e-13, atol=1e-14 * np.abs(ref).max(), err_msg=name)


def test_neighbours_bit_exact(solved):
    name, fx, prob = solved
    if fx["config"].get("local_weight", 1) >= 0.999:
        pytest.skip("local model: no neighbour search")
    assert np.array_equal(prob.get("neigh_offsets"), fx["neigh_offsets"])
    assert np.array_equal(prob.get("neigh_list"), fx["neigh_list"])
    assert prob.scalar("search_radius") == pytest.approx(float(fx["search_radius"][0]), rel=1e-15)


@pytest.mark.parametrize("mat", ["K_inner", "K_bound", "K_local"])
def test_matrix(solved, mat):
    _, fx, prob = solved
    if mat + "_rowptr" not in fx:
        pytest.skip("the radiation branch assembles no separate local matrix")
    rp, ci, va = prob.csr(mat)
    if gc.neumann(fx) and mat != "K_bound":
        rp, ci, va = gc.bordered(rp, ci, va, gc.lagrange_column(fx))
    elif gc.neumann(fx):
        rp = np.zeros(rp.shape[0] + 1, dtype=np.int64)
    assert np.array_equal(rp, fx[mat + "_rowptr"]), "row pointers"
    assert np.array_equal(ci, fx[mat + "_col"]), "column indices"
    ref = fx[mat + "_val"]
    scale = np.abs(ref).max() if ref.size else 1.0
    np.testing.assert_allclose(va, ref, rtol=1e-12, atol=1e-12 * scale)


def test_right_hand_side(solved):
    _, fx, prob = solved
    for name in ["rhs_init", "rhs"]:
        ref = fx[name]
        got = prob.get(name)
        if gc.neumann(fx):   # the Lagrange row's right-hand side is the energy
            got = np.append(got, gc.stationary_parameters(fx["config"])["energy"])
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * max(np.abs(ref).max(), 1.0))
    assert np.array_equal(prob.get("is_inner").astype(np.uint8), fx["is_inner"])


def test_solution(solved):
    _, fx, prob = solved
    if "K_local_rowptr" in fx:   # the linear branches solve with the ILLT
        assert prob.scalar("ilt_ok") == 1
    else:                        # the radiation loop stops after as many steps as the reference's
        assert prob.scalar("nonlinear_iterations") >= 2
    assert rel(prob.get("solution"), fx["temperature"]) < 1e-10


FLUX_RTOL = 1e-12


def assert_flux(got, fx):
    """Both components within 1e-12 of the flux's largest component (a
    component that vanishes in exact arithmetic holds only rounding noise)."""
    scale = max(np.abs(fx["flux_x"]).max(), np.abs(fx["flux_y"]).max(), 1e-300)
    for g, key in zip(got, ("flux_x", "flux_y")):
        np.testing.assert_allclose(g, fx[key], rtol=FLUX_RTOL, atol=FLUX_RTOL * scale, err_msg=key)


def test_flux(solved):
    """heat_equation_solution_2d::calc_flux of the reference's own temperature:
    nodal flux within 1e-12 (max-norm scaled) of the reference's."""
    _, fx, prob = solved
    assert_flux(prob.calc_flux(fx["temperature"]), fx)


def test_flux_variable_conductivity():
    fx = gc.load("b10_field_nonsym")
    prob = gc.oracle_problem(fx)
    prob.set_conductivity_field(fx["conductivity_q"])
    prob.find_neighbours()
    assert_flux(prob.calc_flux(fx["temperature"]), fx)


@pytest.mark.parametrize("name", gc.STATIONARY_2D + ["b10_field_nonsym"])
def test_cuthill_mckee(name):
    """mesh::utils::cuthill_mckee of the mesh as read (before any renumbering):
    every stored variant (local / nonlocal graph, plain / reverse) bit-exact."""
    import oracle
    fx = gc.load(name)
    nodes, elements = gc.mesh_before_renumbering(fx)
    prob = oracle.Problem(gc.element_type(fx), nodes, elements)
    prob.set_model(**gc.model(fx["config"]))
    if fx["config"].get("local_weight", 1) < 0.999:
        prob.find_neighbours(fx["config"].get("strategy", "MAX"))
    variants = [k for k in gc.CUTHILL_MCKEE if k in fx]
    assert variants
    for key in variants:
        assert np.array_equal(prob.cuthill_mckee(*gc.CUTHILL_MCKEE[key]), fx[key]), key


def test_renumbered_mesh_is_the_permuted_mesh():
    """The renumbered fixtures hold mesh_2d::renumbering's result: node i moved
    to permutation[i], elements mapped through the permutation."""
    for name in ("b12_shuffled_cm", "s5_shuffled_cm"):
        fx = gc.load(name)
        nodes, elements = gc.mesh_before_renumbering(fx)
        p = fx["cm_" + fx["config"]["renumber"]]
        assert np.array_equal(fx["nodes"][p], nodes)
        assert np.array_equal(fx["elements"], p[elements])


def test_nonsymmetric_field_matrices():
    """Variable conductivity with a nonlocal model: the oracle reproduces the reference's
    full (non-symmetric) storage bit for bit in pattern and to 1e-12 in values."""
    fx = gc.load("b10_field_nonsym")
    prob = gc.oracle_problem(fx)
    prob.set_conductivity_field(fx["conductivity_q"])
    prob.find_neighbours()
    prob.assemble()
    assert np.array_equal(prob.get("neigh_list"), fx["neigh_list"])
    for mat in ("K_inner", "K_bound"):
        rp, ci, va = prob.csr(mat)
        assert np.array_equal(rp, fx[mat + "_rowptr"]) and np.array_equal(ci, fx[mat + "_col"]), mat
        ref = fx[mat + "_val"]
        np.testing.assert_allclose(va, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(prob.get("rhs"), fx["rhs"], rtol=1e-12, atol=1e-12 * np.abs(fx["rhs"]).max())
    # the fixture's solution solves the full system
    n = fx["K_inner_rowptr"].shape[0] - 1
    a = gc.csr_to_dense(fx["K_inner_rowptr"], fx["K_inner_col"], fx["K_inner_val"], n, n)
    assert not np.allclose(a, a.T)
    assert np.linalg.norm(a @ fx["temperature"] - fx["rhs"]) <= 1e-12 * np.linalg.norm(fx["rhs"])
    # the oracle's own BiCGSTAB reaches the reference's solution
    prob.solve(tol=1e-13, maxit=20000)
    t = prob.get("solution")
    assert np.linalg.norm(t - fx["temperature"]) <= 1e-10 * np.linalg.norm(fx["temperature"])


def test_known_answers():
    """The reference's own analytic checks, on the oracle's solution."""
    fx = gc.load("ref_square16_manufactured")
    prob = gc.oracle_problem(fx)
    prob.find_neighbours()
    prob.assemble(); prob.assemble_local(); prob.solve(tol=1e-14)
    t, ex = prob.get("solution"), fx["exact_solution"]
    assert ((t - ex) ** 2).sum() / (ex ** 2).sum() < 1e-3          # boundary_conditions_2d.cpp:111
    fx = gc.load("ref_solid_ring")
    prob = gc.oracle_problem(fx)
    prob.find_neighbours()
    prob.assemble(); prob.assemble_local(); prob.solve(tol=1e-14)
    x = fx["nodes"]
    exact = 1.0 + np.log(np.hypot(x[:, 0], x[:, 1])) / np.log(2.0)
    err = np.abs(prob.get("solution") - exact).max() / np.abs(exact).max()
    assert err < 1.4e-3                                             # isotropic_solid_ring.cpp:43-45


def test_ic0_variant_converges_to_same_solution():
    fx = gc.load("s6_exp_ortho_jitter")
    prob = gc.oracle_problem(fx)
    prob.find_neighbours()
    prob.assemble(); prob.assemble_local()
    prob.solve(variant=1, tol=1e-14)
    assert prob.scalar("ilt_ok") == 1
    assert rel(prob.get("solution"), fx["temperature"]) < 1e-10


def test_nonstationary_history():
    import oracle
    fx = gc.load("b8_nonstationary")
    cfg = fx["config"]
    prob = oracle.Problem(gc.element_type(fx), fx["nodes"], fx["elements"])
    prob.set_model(**gc.model(cfg))
    prob.add_boundary(0, fx["bnd_" + cfg["dirichlet_group"]], 0.0)
    prob.find_neighbours()
    prob.nonstationary(float(cfg["dt"]), int(cfg["steps"]), float(cfg["omega"]))
    hist = prob.get("history").reshape(int(cfg["steps"]), -1)
    ref = fx["temperature_history"]
    for s in range(hist.shape[0]):
        assert rel(hist[s], ref[s]) < 1e-10, s


@pytest.mark.parametrize("name", ["d1_quadratic_1000", "d1_linear_40_triangle"])
def test_stationary_1d(name):
    import oracle
    fx = gc.load(name)
    cfg = fx["config"]
    t = oracle.stationary_1d(elements=int(cfg["elements"]), order=int(cfg["order"]), radius=float(cfg["radius"]),
                             local_weight=float(cfg["local_weight"]), influence=cfg["influence"],
                             conductivity=float(cfg["conductivity"]), t_left=float(cfg["left_temperature"]),
                             q_right=float(cfg["right_flux"]), sin_source=cfg["source"] == "sin")
    assert rel(t, fx["temperature"]) < 1e-10


@pytest.mark.parametrize("name", ["m8_mechanical", "s4_mechanical_local"])
def test_mechanical_fixtures(name):
    """The reference's plane-elasticity runs (DoF = 2): stiffness rows per node and
    degree of freedom in upper storage, clamped degrees of freedom as unit rows,
    and a displacement that solves the stored system."""
    fx = gc.load(name)
    n = fx["nodes"].shape[0]
    rp, ci, va = fx["K_inner_rowptr"], fx["K_inner_col"], fx["K_inner_val"]
    assert rp.shape[0] == 2 * n + 1
    rows = np.repeat(np.arange(2 * n), np.diff(rp))
    assert np.all(ci >= rows)
    clamped = np.flatnonzero(fx["is_inner"] == 0)
    for r in clamped:
        assert rp[r + 1] - rp[r] == 1 and ci[rp[r]] == r and va[rp[r]] == 1.0
    a = gc.csr_to_dense(rp, ci, va, 2 * n, 2 * n)
    a = a + np.triu(a, 1).T
    u, f = fx["displacement"], fx["rhs"]
    assert np.linalg.norm(a @ u - f) <= 1e-12 * np.linalg.norm(f)
    assert np.allclose(u[clamped], 0.0)
