"""Parity of the CUDA path (through the C ABI) with the reference.

* golden fixtures: the reference's own outputs on the same inputs
  (tests/golden, made by tests/golden/make_golden.py): neighbour lists and
  sparsity patterns bit-exact, matrix values and right-hand sides within
  1e-12 relative (max-norm scaled), nodal temperature within 1e-10 relative L2;
* the oracle (CPU restatement pinned to those fixtures) on larger cases of the
  benchmark shapes with the same r/h;
* size-independent properties at the full benchmark sizes.
"""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

MATRIX_RTOL = 1e-12
SOLUTION_RTOL = 1e-10


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.fixture(scope="session")
def lib():
    from nonlocal_gb300 import _lib, build
    build.build()
    _lib.load()
    if _lib.device_count() == 0:
        pytest.fail("no CUDA device visible to the nlgpu library")
    return _lib


def gpu_problem(fx):
    from nonlocal_gb300 import thermal as T
    cfg = fx["config"]
    pb = T.Problem2D(gc.element_type(fx), fx["nodes"], fx["elements"])
    m = gc.model(cfg)
    kind, cond = m["cond_kind"], m["cond"]
    pb.set_model(T.Model2D(influence={v: k for k, v in gc.INFLUENCE.items()}[m["influence"]], radius=m["radius"],
                           local_weight=m["local_weight"], n=m["n"], p=m["p"], q=m["q"],
                           conductivity=cond[:kind + 1]))
    for d in gc.boundary_specs(fx):
        pb.add_boundary(T.Boundary(**d))
    pb.set_stationary_parameters(**gc.stationary_parameters(cfg))
    if cfg.get("source") == "manufactured":
        pb.set_source(0.0, fx["source_q"])
    elif "source" in cfg:
        pb.set_source(float(cfg["source"]))
    if "dirichlet_values" in fx:
        pb.set_dirichlet_values(fx["dirichlet_values"])
    return pb


def assert_csr_equal(got, fx, name):
    rp, col, val = got
    assert np.array_equal(rp, fx[name + "_rowptr"]), f"{name}: row pointers"
    assert np.array_equal(col, fx[name + "_col"]), f"{name}: columns"
    ref = fx[name + "_val"]
    scale = np.abs(ref).max() if ref.size else 1.0
    np.testing.assert_allclose(val, ref, rtol=MATRIX_RTOL, atol=MATRIX_RTOL * scale, err_msg=name)


@pytest.fixture(scope="module", params=gc.STATIONARY_2D)
def golden(request, lib):
    fx = gc.load(request.param)
    pb = gpu_problem(fx)
    return request.param, fx, pb


def test_basis_and_quadrature(golden):
    _, fx, pb = golden
    b = pb.basis()
    for k, v in b.items():
        np.testing.assert_allclose(v, fx[k].reshape(-1), rtol=0, atol=2e-15, err_msg=k)
    qc, jac, der = pb.quadrature()
    for got, key in [(qc, "qcoords"), (jac, "jacobians"), (der, "derivatives")]:
        ref = fx[key].reshape(-1)
        np.testing.assert_allclose(got.reshape(-1), ref, rtol=1e-13, atol=1e-14 * np.abs(ref).max(), err_msg=key)


def test_neighbours_bit_exact(golden):
    name, fx, pb = golden
    if fx["config"].get("local_weight", 1) >= 0.999:
        pytest.skip("local model")
    r, pairs = pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    off, lst = pb.neighbours()
    assert r[0] == pytest.approx(float(fx["search_radius"][0]), rel=1e-15)
    assert np.array_equal(off, fx["neigh_offsets"])
    assert np.array_equal(lst, fx["neigh_list"])


def test_matrices_and_rhs(golden):
    _, fx, pb = golden
    if fx["config"].get("local_weight", 1) < 0.999:
        pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    pb.conductivity_matrix("FULL")
    assert_csr_equal(pb.matrix("inner"), fx, "K_inner")
    assert_csr_equal(pb.matrix("bound"), fx, "K_bound")
    f, f0 = pb.rhs()
    for got, key in [(f0, "rhs_init"), (f, "rhs")]:
        np.testing.assert_allclose(got, fx[key], rtol=MATRIX_RTOL, atol=MATRIX_RTOL * max(np.abs(fx[key]).max(), 1.0))
    if "K_local_rowptr" in fx:   # the radiation branch assembles no separate local matrix
        pb.conductivity_matrix("LOCAL")
        assert_csr_equal(pb.matrix("local"), fx, "K_local")


def test_float_float_assembly_matrices(golden):
    """The mixed-precision form's pair blocks, computed in float-float on the FP32
    pipes, meet the FP64 entries' bar against the reference's matrices (models
    outside its scope run the FP64 kernel and pass trivially)."""
    _, fx, pb = golden
    if fx["config"].get("local_weight", 1) < 0.999:
        pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    pb.set_assembly_precision("ff")
    try:
        pb.conductivity_matrix("FULL")
        assert_csr_equal(pb.matrix("inner"), fx, "K_inner")
        assert_csr_equal(pb.matrix("bound"), fx, "K_bound")
    finally:
        pb.set_assembly_precision("auto")


@pytest.mark.parametrize("warps", [16, 32])
def test_float_float_assembly_warps(golden, warps):
    """Both CTA shapes of the float-float pair assembly (16 and 32 warps, which
    the tuner chooses between) meet the FP64 bar against the reference's
    matrices, and the tuner reports one of them."""
    _, fx, pb = golden
    if fx["config"].get("local_weight", 1) < 0.999:
        pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    pb.set_assembly_precision("ff")
    try:
        pb.set_assembly_warps(warps)
        pb.conductivity_matrix("FULL")
        assert_csr_equal(pb.matrix("inner"), fx, "K_inner")
        assert_csr_equal(pb.matrix("bound"), fx, "K_bound")
        tuning = pb.assembly_tuning()
        assert tuning["warps"] in (0, warps)   # 0: the model runs the FP64 kernel
        pb.set_assembly_warps(0)
        pb.conductivity_matrix("FULL")
        assert_csr_equal(pb.matrix("inner"), fx, "K_inner")
        assert pb.assembly_tuning()["warps"] in (0, 16, 32)
    finally:
        pb.set_assembly_warps(0)
        pb.set_assembly_precision("auto")


def test_stationary_solution(golden):
    _, fx, pb = golden
    if fx["config"].get("local_weight", 1) < 0.999:
        pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    t, rep = pb.stationary(tolerance=1e-13, max_iterations=20000)
    assert rep.preconditioner_ok == 1
    assert rep.residual <= 1e-13
    assert rel(t, fx["temperature"]) < SOLUTION_RTOL


def test_nonsymmetric_variable_conductivity(lib):
    """A spatially varying conductivity with a nonlocal model makes the reference's
    system non-symmetric (full storage) and solved by BiCGSTAB: same neighbours,
    patterns, values, right-hand side and solution."""
    fx = gc.load("b10_field_nonsym")
    pb = gpu_problem(fx)
    pb.set_conductivity_field(fx["conductivity_q"])
    pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    off, lst = pb.neighbours()
    assert np.array_equal(off, fx["neigh_offsets"]) and np.array_equal(lst, fx["neigh_list"])
    pb.conductivity_matrix("FULL")
    assert_csr_equal(pb.matrix("inner"), fx, "K_inner")
    assert_csr_equal(pb.matrix("bound"), fx, "K_bound")
    rp = fx["K_inner_rowptr"]
    assert rp[-1] > 2 * (rp.shape[0] - 1) and np.any(np.diff(rp) > 20)   # full rows, not the upper half
    f, _ = pb.rhs()
    np.testing.assert_allclose(f, fx["rhs"], rtol=MATRIX_RTOL, atol=MATRIX_RTOL * np.abs(fx["rhs"]).max())
    t, rep = pb.solve_assembled(tolerance=1e-13, max_iterations=20000)
    assert rep.residual <= 1e-13
    assert rel(t, fx["temperature"]) < SOLUTION_RTOL
    assert_flux(pb.calc_flux(fx["temperature"]), fx)
    # the ordered pairs in float-float on the FP32 pipes meet the same bar
    pb.set_assembly_precision("ff")
    try:
        pb.conductivity_matrix("FULL")
        assert pb.assembly_tuning()["warps"] in (16, 32)
        assert_csr_equal(pb.matrix("inner"), fx, "K_inner")
        assert_csr_equal(pb.matrix("bound"), fx, "K_bound")
        t, rep = pb.solve_assembled(tolerance=1e-13, max_iterations=20000)
        assert rel(t, fx["temperature"]) < SOLUTION_RTOL
    finally:
        pb.set_assembly_precision("auto")


def test_batched_nonsymmetric_solves_match_single_instances(lib):
    """nlgpu_solve_assembled_batch: the reference's variable-conductivity
    fixture and log-normal-conductivity instances of uneven size, radius and
    p1 solved as one block-diagonal BiCGSTAB reach the fixture's temperature
    and each instance's single-system BiCGSTAB solution; a symmetric instance
    in the same call is solved on its own."""
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.fields import lognormal_conductivity
    from nonlocal_gb300.meshgen import structured_quad_mesh
    fx = gc.load("b10_field_nonsym")
    problems = []
    pb = gpu_problem(fx)
    pb.set_conductivity_field(fx["conductivity_q"])
    pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    problems.append(pb)
    for k, (nx, r, p1) in enumerate([(12, 0.2, 0.3), (20, 0.08, 0.7), (16, 0.12, 0.5)]):
        mesh = structured_quad_mesh(nx, nx, "bilinear")
        q = T.Problem2D.from_mesh(mesh)
        q.set_model(T.Model2D(influence="fast_polynomial", radius=(r, r), local_weight=p1))
        q.set_conductivity_field(lognormal_conductivity(q.quadrature()[0], 0.1, 0.5, seed=k))
        q.add_boundary(T.Boundary(edges=mesh.boundaries["left"], kind="temperature", value=0.0))
        q.add_boundary(T.Boundary(edges=mesh.boundaries["right"], kind="flux", value=1.0))
        q.find_neighbours()
        problems.append(q)
    mesh = structured_quad_mesh(10, 10, "bilinear")
    sym = T.Problem2D.from_mesh(mesh)
    sym.set_model(T.Model2D(influence="fast_polynomial", radius=(0.2, 0.2), local_weight=0.5))
    sym.add_boundary(T.Boundary(edges=mesh.boundaries["left"], kind="temperature", value=0.0))
    sym.add_boundary(T.Boundary(edges=mesh.boundaries["right"], kind="flux", value=1.0))
    sym.find_neighbours()
    problems.insert(2, sym)
    for q in problems:
        q.conductivity_matrix("FULL")
    temps, reps = T.solve_assembled_batch(problems, tolerance=1e-13, max_iterations=20000)
    for t, rep in zip(temps, reps):
        assert rep.residual <= 1e-13 and rep.iterations > 0
    assert rel(temps[0], fx["temperature"]) < SOLUTION_RTOL
    for q, t in zip(problems, temps):
        single, rep = q.solve_assembled(tolerance=1e-13, max_iterations=20000)
        assert rel(t, single) < 1e-9   # two solutions with |b - Ax| <= 1e-13 |b| each
    # MIXED: the FP32 ILLT of each local part instead of the diagonal, batched and alone
    temps_m, reps_m = T.solve_assembled_batch(problems, tolerance=1e-13, max_iterations=20000, precision="mixed")
    assert rel(temps_m[0], fx["temperature"]) < SOLUTION_RTOL
    for k, (q, t, tm, rep, rep_m) in enumerate(zip(problems, temps, temps_m, reps, reps_m)):
        assert rep_m.residual <= 1e-13
        assert rel(tm, t) < 1e-9, k
        if k != 2:   # the non-symmetric ones: fewer iterations than with the diagonal
            assert rep_m.iterations < rep.iterations, (k, rep_m.iterations, rep.iterations)
            single, rep_s = q.solve_assembled(tolerance=1e-13, max_iterations=20000, precision="mixed")
            assert rel(single, t) < 1e-9 and rep_s.residual <= 1e-13
    for q in problems:
        q.close()


FLUX_RTOL = 1e-12


def assert_flux(got, fx):
    """Both components within 1e-12 of the flux's largest component: a
    component that vanishes in exact arithmetic (flux_y of a problem without
    y-dependence) holds rounding noise and is judged on the vector's scale."""
    scale = max(np.abs(fx["flux_x"]).max(), np.abs(fx["flux_y"]).max(), 1e-300)
    for g, key in zip(got, ("flux_x", "flux_y")):
        np.testing.assert_allclose(g, fx[key], rtol=FLUX_RTOL, atol=FLUX_RTOL * scale, err_msg=key)


def test_flux(golden):
    """heat_equation_solution_2d::calc_flux of the reference's temperature: the
    nodal flux within 1e-12 (max-norm scaled) of the reference's own."""
    _, fx, pb = golden
    assert_flux(pb.calc_flux(fx["temperature"]), fx)


def test_mixed_precision_solution(golden):
    """FP32 inner flexible CG + FP64 refinement reaches the reference's FP64 solution:
    the FP64 residual decides convergence, so the bar is the plain one."""
    _, fx, pb = golden
    if fx["config"].get("local_weight", 1) < 0.999:
        pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    # ILLT applied by Jacobi sweeps (the default) and by exact level-scheduled sweeps,
    # and with the coarse-space correction over about 16 aggregates
    for pre, sweeps, coarse in (("illt", 0, 0), ("illt", -1, 0), ("identity", 0, 0), ("illt", 0, 16)):
        t, rep = pb.stationary(tolerance=1e-13, max_iterations=50000, preconditioner=pre, precision="mixed",
                               triangular_sweeps=sweeps, coarse_aggregates=coarse)
        assert rep.residual <= 1e-13
        assert rep.outer_iterations >= 1 and rep.iterations > 0
        assert rel(t, fx["temperature"]) < SOLUTION_RTOL, (pre, sweeps, coarse)


@pytest.mark.parametrize("shape", ["bilinear", "serendipity"])
def test_coarse_correction_cuts_iterations(lib, shape):
    """The coarse-space correction (aggregates of about 8 x 8 elements) reaches the
    plain FP64 solution of a 64 x 64 nonlocal problem (config-2 / config-3 shapes
    scaled, r / h kept near the benchmark's) in far fewer FCG iterations than
    ILLT alone, with the FP64 residual deciding convergence."""
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    if shape == "bilinear":
        mesh = structured_quad_mesh(64, 64, "bilinear")
        model = T.Model2D(influence="fast_polynomial", radius=(0.16, 0.16), local_weight=0.5)
        bcs = [("left", "temperature", 0.0), ("right", "flux", 1.0)]
    else:
        mesh = structured_quad_mesh(64, 64, "serendipity", jitter=0.2, seed=0)
        model = T.Model2D(influence="exponential", radius=(0.1, 0.1), local_weight=0.3, conductivity=(1.0, 0.1))
        bcs = [("up", "temperature", 1.0), ("down", "temperature", 0.0)]
    pb = T.Problem2D.from_mesh(mesh)
    pb.set_model(model)
    for g, kind, v in bcs:
        pb.add_boundary(T.Boundary(edges=mesh.boundaries[g], kind=kind, value=v))
    pb.find_neighbours()
    ref, _ = pb.stationary(tolerance=1e-13, max_iterations=20000)
    t0, rep0 = pb.stationary(tolerance=1e-12, max_iterations=20000, precision="mixed")
    t1, rep1 = pb.stationary(tolerance=1e-12, max_iterations=20000, precision="mixed", coarse_aggregates=64)
    assert rep1.residual <= 1e-12 and rep0.residual <= 1e-12
    assert rel(t1, ref) < 1e-9 and rel(t0, ref) < 1e-9
    assert rep1.iterations * 2 < rep0.iterations, (rep1.iterations, rep0.iterations)


@pytest.mark.parametrize("name", ["b12_fastpoly", "s6_exp_ortho_jitter"])
def test_symmetric_fp32_spmv(lib, name):
    """The mixed solve with the FP32 SpMV reading only the strictly upper part
    (NLGPU_OPTION_FP32_SYMMETRIC, shared-memory scatter of the transposed
    entries) reaches the reference's solution like the full-row SpMV, with the
    same iteration count up to the order of its atomic additions."""
    fx = gc.load(name)
    runs = []
    for symmetric in (0, 1):
        pb = gpu_problem(fx)
        lib.check(lib.load().nlgpu_set_option(pb.handle, lib.OPTION_FP32_SYMMETRIC, symmetric))
        if fx["config"].get("local_weight", 1) < 0.999:
            pb.find_neighbours(fx["config"].get("strategy", "MAX"))
        t, rep = pb.stationary(tolerance=1e-13, max_iterations=50000, precision="mixed")
        assert rep.fp32_symmetric == symmetric
        assert rep.nnz_fp32 == (rep.nnz_inner - pb.n_nodes if symmetric else rep.nnz_solver)
        assert rel(t, fx["temperature"]) < SOLUTION_RTOL, symmetric
        runs.append(rep.iterations)
    assert abs(runs[0] - runs[1]) <= max(3, runs[0] // 20), runs


@pytest.mark.parametrize("name", ["b12_fastpoly", "s6_exp_ortho_jitter"])
def test_tma_sweeps_match_global_sweeps(lib, name):
    """The TMA-fed shared-memory triangular sweeps compute what the global-memory
    sweeps compute (same entries in the same order; the two assemblies differ
    only by the order of atomic additions)."""
    fx = gc.load(name)
    runs = []
    for global_sweeps in (0, 1):
        pb = gpu_problem(fx)
        lib.check(lib.load().nlgpu_set_option(pb.handle, 0, global_sweeps))
        pb.find_neighbours()
        t, rep = pb.stationary(tolerance=1e-12)
        runs.append((t, rep.iterations))
    assert abs(runs[0][1] - runs[1][1]) <= 1
    assert rel(runs[0][0], runs[1][0]) < 1e-12


def test_known_answers(lib):
    fx = gc.load("ref_square16_manufactured")
    t, _ = gpu_problem(fx).stationary(tolerance=1e-13)
    ex = fx["exact_solution"]
    assert ((t - ex) ** 2).sum() / (ex ** 2).sum() < 1e-3                # boundary_conditions_2d.cpp:111
    fx = gc.load("ref_solid_ring")
    t, _ = gpu_problem(fx).stationary(tolerance=1e-13)
    x = fx["nodes"]
    exact = 1.0 + np.log(np.hypot(x[:, 0], x[:, 1])) / np.log(2.0)
    assert np.abs(t - exact).max() / np.abs(exact).max() < 1.4e-3        # isotropic_solid_ring.cpp:43-45


def test_cg_on_reference_matrices(lib):
    """slae::conjugate_gradient with ILLT(p1 K_local) on the reference's own matrices."""
    from nonlocal_gb300 import thermal as T
    fx = gc.load("s6_exp_ortho_jitter")
    ctx = gpu_problem(fx)
    a = (fx["K_inner_rowptr"], fx["K_inner_col"], fx["K_inner_val"])
    p = (fx["K_local_rowptr"], fx["K_local_col"], fx["K_local_val"])
    x, rep = T.conjugate_gradient(ctx, a, fx["rhs"], preconditioner_csr=p, tolerance=1e-13)
    assert rep.preconditioner_ok == 1
    assert rel(x, fx["temperature"]) < SOLUTION_RTOL
    x2, rep2 = T.conjugate_gradient(ctx, a, fx["rhs"], tolerance=1e-13)     # identity preconditioner
    assert rel(x2, fx["temperature"]) < SOLUTION_RTOL
    assert rep2.iterations > rep.iterations


def test_illt_preconditioner_plugin(lib):
    """The ILLT behind preconditioner_base: exact on a matrix without fill, symmetric
    and positive on the reference's local matrix."""
    from nonlocal_gb300 import thermal as T
    # tridiagonal SPD: IC(0) has no dropped fill, so M^-1 = A^-1 (the first attempt
    # uses no shift because the scaled diagonal is positive)
    n = 500
    rp = np.arange(0, 2 * n, 2, dtype=np.int64)
    rp = np.append(rp, 2 * n - 1)
    col = np.empty(2 * n - 1, dtype=np.int64)
    val = np.empty(2 * n - 1)
    col[0::2] = np.arange(n)
    col[1::2] = np.arange(1, n)
    val[0::2] = 2.0 + 0.01 * np.arange(n) / n
    val[1::2] = -1.0
    pre = T.EigenILLTPreconditioner()
    assert pre.compute((rp, col, val)).computation_info() == pre.SUCCESS
    dense = gc.csr_to_dense(rp, col, val, n, n)
    dense = dense + np.triu(dense, 1).T
    b = np.sin(np.arange(n) * 0.37)
    assert rel(pre.solve(b), np.linalg.solve(dense, b)) < 1e-12

    fx = gc.load("s6_exp_ortho_jitter")
    p = (fx["K_local_rowptr"], fx["K_local_col"], fx["K_local_val"])
    m = fx["K_local_rowptr"].shape[0] - 1
    assert pre.compute(p).computation_info() == pre.SUCCESS
    rng = np.random.default_rng(3)
    a, c = rng.standard_normal(m), rng.standard_normal(m)
    ma, mc = pre.solve(a), pre.solve(c)
    assert abs(ma @ c - a @ mc) <= 1e-10 * np.linalg.norm(ma) * np.linalg.norm(c)
    assert ma @ a > 0 and mc @ c > 0
    assert np.array_equal(pre.solve(a), ma)   # deterministic


def test_nonstationary_history(lib):
    from nonlocal_gb300 import thermal as T
    fx = gc.load("b8_nonstationary")
    cfg = fx["config"]
    pb = T.Problem2D(gc.element_type(fx), fx["nodes"], fx["elements"])
    m = gc.model(cfg)
    pb.set_model(T.Model2D(influence="fast_polynomial", radius=m["radius"], local_weight=m["local_weight"]))
    pb.add_boundary(T.Boundary(edges=fx["bnd_" + cfg["dirichlet_group"]], kind="temperature", value=0.0))
    dt, steps, omega = float(cfg["dt"]), int(cfg["steps"]), float(cfg["omega"])
    solver = T.NonstationaryHeatEquationSolver2D(pb, dt)
    solver.compute()
    for s in range(1, steps + 1):
        t = solver.calc_step(np.sin(omega * s * dt), tolerance=1e-15, max_iterations=10000)
        assert rel(t, fx["temperature_history"][s - 1]) < SOLUTION_RTOL, s


def test_nonstationary_history_with_radiation(lib):
    """Flux, convection and radiation on one side of a nonstationary problem: the
    convection matrix scaled by dt at compute, and each step's radiation terms
    (dt 4 sigma eps int T^3 N_i N_j kept in the matrix, 3 sigma eps int T^4 N_i in
    the right-hand side), against the reference's 5-step history."""
    from nonlocal_gb300 import thermal as T
    fx = gc.load("b8_nonstationary_radiation")
    cfg = fx["config"]
    pb = T.Problem2D(gc.element_type(fx), fx["nodes"], fx["elements"])
    m = gc.model(cfg)
    pb.set_model(T.Model2D(influence="fast_polynomial", radius=m["radius"], local_weight=m["local_weight"]))
    pb.add_boundary(T.Boundary(edges=fx["bnd_" + cfg["dirichlet_group"]], kind="temperature", value=0.0))
    for d in gc.boundary_specs(fx):
        pb.add_boundary(T.Boundary(**d))
    dt, steps, omega = float(cfg["dt"]), int(cfg["steps"]), float(cfg["omega"])
    solver = T.NonstationaryHeatEquationSolver2D(pb, dt)
    solver.compute(np.full(pb.n_nodes, float(cfg["initial"])))
    for s in range(1, steps + 1):
        t = solver.calc_step(np.sin(omega * s * dt), tolerance=1e-15, max_iterations=10000)
        assert rel(t, fx["temperature_history"][s - 1]) < SOLUTION_RTOL, s


def test_batched_nonstationary_matches_single_instances(lib):
    """Instances of different sizes, radii and time steps stepped as one batch give
    the temperatures (and iteration counts) of stepping each on its own."""
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    specs = [(12, 0.25, 1e-3), (20, 0.15, 1e-3), (9, 0.3, 2e-3), (16, 0.2, 5e-4)]

    def build(nx, r, dt):
        mesh = structured_quad_mesh(nx, nx, "bilinear")
        pb = T.Problem2D.from_mesh(mesh)
        pb.set_model(T.Model2D(influence="fast_polynomial", radius=(r, r), local_weight=0.5))
        pb.add_boundary(T.Boundary(edges=mesh.boundaries["left"], kind="temperature", value=0.0))
        pb.add_boundary(T.Boundary(edges=mesh.boundaries["right"], kind="flux", value=1.0))
        s = T.NonstationaryHeatEquationSolver2D(pb, dt)
        s.compute()
        return s

    singles = [build(*sp) for sp in specs]
    batched = [build(*sp) for sp in specs]
    batch = T.BatchNonstationary(batched)
    for step in range(1, 6):
        values = [np.sin(10.0 * step * sp[2]) for sp in specs]
        its = batch.step(values, tolerance=1e-13, max_iterations=5000)
        for k, s in enumerate(singles):
            t = s.calc_step(values[k], tolerance=1e-13, max_iterations=5000)
            assert rel(batch.temperature(k), t) < SOLUTION_RTOL, (step, k)
            assert abs(int(its[k]) - s.iterations[-1]) <= 2, (step, k, its[k], s.iterations[-1])
    batch.close()


def test_batched_mixed_illt_matches_single_instances(lib):
    """The batched step's mixed-precision ILLT method (FCG on the whole
    block-diagonal system, FP64 reliable updates, every instance held to its own
    relative residual) reaches the temperatures of the reference's identity FP64
    CG stepping each instance on its own, in fewer iterations."""
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    specs = [(12, 0.25, 1e-3), (20, 0.15, 1e-3), (9, 0.3, 2e-3), (16, 0.2, 5e-4)]

    def build(nx, r, dt):
        mesh = structured_quad_mesh(nx, nx, "bilinear")
        pb = T.Problem2D.from_mesh(mesh)
        pb.set_model(T.Model2D(influence="fast_polynomial", radius=(r, r), local_weight=0.5))
        pb.add_boundary(T.Boundary(edges=mesh.boundaries["left"], kind="temperature", value=0.0))
        pb.add_boundary(T.Boundary(edges=mesh.boundaries["right"], kind="flux", value=1.0))
        s = T.NonstationaryHeatEquationSolver2D(pb, dt)
        s.compute()
        return s

    singles = [build(*sp) for sp in specs]
    batch = T.BatchNonstationary([build(*sp) for sp in specs])
    batch.set_method("mixed_illt")
    for step in range(1, 6):
        values = [np.sin(10.0 * step * sp[2]) for sp in specs]
        its = batch.step(values, tolerance=1e-13, max_iterations=5000)
        for k, s in enumerate(singles):
            t = s.calc_step(values[k], tolerance=1e-13, max_iterations=5000)
            assert rel(batch.temperature(k), t) < SOLUTION_RTOL, (step, k)
        assert int(its.max()) < max(s.iterations[-1] for s in singles), (step, its, [s.iterations[-1] for s in singles])
    batch.close()


@pytest.mark.parametrize("name", ["d1_quadratic_1000", "d1_linear_40_triangle"])
def test_stationary_1d(lib, name):
    from nonlocal_gb300 import thermal as T
    fx = gc.load(name)
    cfg = fx["config"]
    t = T.stationary_heat_equation_solver_1d(elements=int(cfg["elements"]), order=int(cfg["order"]),
                                             radius=float(cfg["radius"]), local_weight=float(cfg["local_weight"]),
                                             influence=cfg["influence"], conductivity=float(cfg["conductivity"]),
                                             t_left=float(cfg["left_temperature"]), q_right=float(cfg["right_flux"]),
                                             sin_source=cfg["source"] == "sin")
    assert rel(t, fx["temperature"]) < SOLUTION_RTOL


# ---------------------------------------------------------------- oracle, larger cases
def oracle_and_gpu(mesh, model_kw, bcs, lib):
    import oracle
    from nonlocal_gb300 import thermal as T
    et = 2 if mesh.element == "bilinear" else 3
    prob = oracle.Problem(et, mesh.nodes, mesh.elements)
    kind = {1: 0, 2: 1, 3: 2}[len(model_kw["conductivity"])]
    prob.set_model(influence=gc.INFLUENCE[model_kw["influence"]], n=2, p=model_kw.get("p", 2),
                   q=model_kw.get("q", 0.5 if model_kw["influence"] == "exponential" else 1.0),
                   radius=model_kw["radius"], local_weight=model_kw["local_weight"], cond_kind=kind,
                   cond=tuple(model_kw["conductivity"]) + (0.0,) * (3 - len(model_kw["conductivity"])))
    pb = T.Problem2D.from_mesh(mesh)
    pb.set_model(T.Model2D(**model_kw))
    for group, kind_, value in bcs:
        prob.add_boundary(0 if kind_ == "temperature" else 1, mesh.boundaries[group], value)
        pb.add_boundary(T.Boundary(edges=mesh.boundaries[group], kind=kind_, value=value))
    return prob, pb


@pytest.mark.parametrize("case", ["config2_scaled_40", "config3_scaled_20"])
def test_against_oracle_scaled(lib, case):
    from nonlocal_gb300.meshgen import structured_quad_mesh
    if case == "config2_scaled_40":
        mesh = structured_quad_mesh(40, 40, "bilinear")
        model = dict(influence="fast_polynomial", radius=(0.25, 0.25), local_weight=0.5, conductivity=(1.0,))
        bcs = [("left", "temperature", 0.0), ("right", "flux", 1.0)]
    else:
        mesh = structured_quad_mesh(20, 20, "serendipity", jitter=0.2, seed=0)
        model = dict(influence="exponential", radius=(0.15, 0.15), local_weight=0.3, conductivity=(1.0, 0.1))
        bcs = [("up", "temperature", 1.0), ("down", "temperature", 0.0)]
    prob, pb = oracle_and_gpu(mesh, model, bcs, lib)
    prob.find_neighbours()
    prob.assemble()
    prob.assemble_local()
    prob.solve(variant=1, tol=1e-13)
    pb.find_neighbours()
    off, lst = pb.neighbours()
    assert np.array_equal(off, prob.get("neigh_offsets"))
    assert np.array_equal(lst, prob.get("neigh_list"))
    pb.conductivity_matrix("FULL")
    rp, col, val = pb.matrix("inner")
    orp, ocol, oval = prob.csr("K_inner")
    assert np.array_equal(rp, orp) and np.array_equal(col, ocol)
    np.testing.assert_allclose(val, oval, rtol=MATRIX_RTOL, atol=MATRIX_RTOL * np.abs(oval).max())
    # the float-float pair blocks of the mixed-precision form, same bar
    pb.set_assembly_precision("ff")
    pb.conductivity_matrix("FULL")
    np.testing.assert_allclose(pb.matrix("inner")[2], oval, rtol=MATRIX_RTOL, atol=MATRIX_RTOL * np.abs(oval).max())
    pb.set_assembly_precision("auto")
    t, rep = pb.stationary(tolerance=1e-13)
    assert rel(t, prob.get("solution")) < SOLUTION_RTOL
    # same preconditioner (fixed-pattern IC(0) on the scaled, shifted local matrix): iteration counts agree
    assert abs(rep.iterations - prob.scalar("iterations")) <= 2
    # the mixed-precision form against the FP64 oracle solution (Jacobi and exact sweeps)
    for sweeps in (0, -1):
        tm, repm = pb.solve_assembled(tolerance=1e-13, precision="mixed", triangular_sweeps=sweeps)
        assert repm.residual <= 1e-13
        assert rel(tm, prob.get("solution")) < SOLUTION_RTOL, sweeps
    # the nodal flux of the same temperature field (scaled by the flux vector's
    # largest component: a component that nearly cancels keeps the other's scale)
    gx, gy = pb.calc_flux(t)
    ox, oy = prob.calc_flux(t)
    scale = max(np.abs(ox).max(), np.abs(oy).max())
    for g, o in ((gx, ox), (gy, oy)):
        np.testing.assert_allclose(g, o, rtol=FLUX_RTOL, atol=FLUX_RTOL * scale)


def test_illt_jacobi_sweeps(lib):
    """The FP32 ILLT application of the mixed solve: k Jacobi sweeps per triangle
    equal the first k + 1 terms of the Neumann series of each triangular inverse,
    computed here in FP64 from the oracle's factor of the same matrix; exact
    FP32 sweeps and enough Jacobi sweeps (more than the level count) reproduce
    the exact FP64 application."""
    import scipy.sparse as sp
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    mesh = structured_quad_mesh(20, 20, "serendipity", jitter=0.2, seed=0)
    model = dict(influence="exponential", radius=(0.15, 0.15), local_weight=0.3, conductivity=(1.0, 0.1))
    prob, _ = oracle_and_gpu(mesh, model, [("up", "temperature", 1.0), ("down", "temperature", 0.0)], lib)
    prob.find_neighbours()
    prob.assemble()
    prob.assemble_local()
    prob.solve(variant=1, tol=1e-6)   # the fixed-pattern IC(0) factor the CUDA path computes
    rp, col, val = prob.csr("K_local")
    n = rp.shape[0] - 1
    pre = T.EigenILLTPreconditioner()
    assert pre.compute((rp, col, val)).computation_info() == pre.SUCCESS
    u = sp.csr_matrix((prob.get("L_val"), prob.get("L_col"), prob.get("L_rowptr")), shape=(n, n))
    s, d = prob.get("L_scale"), u.diagonal()
    upper = sp.diags(1.0 / d) @ sp.triu(u, 1).tocsr()          # D^-1 N^T
    lower = sp.diags(1.0 / d) @ sp.triu(u, 1).T.tocsr()        # D^-1 N

    def neumann(x, k):
        c = s / d
        y = c * x
        for _ in range(k):
            y = c * x - lower @ y
        yt = y / d
        z = yt.copy()
        for _ in range(k):
            z = yt - upper @ z
        return s * z

    x = np.random.default_rng(5).standard_normal(n)
    for k in (1, 2, 6):
        assert rel(pre.solve_f32(x, k).astype(np.float64), neumann(x, k)) < 2e-5, k
    exact = pre.solve(x)
    assert rel(pre.solve_f32(x, -1).astype(np.float64), exact) < 2e-5
    assert rel(pre.solve_f32(x, n).astype(np.float64), exact) < 1e-4
    assert rel(neumann(x, 6), exact) > 1e-3   # six sweeps are an approximation here


def test_operator_annihilates_constants_full_size(lib):
    """Without boundary conditions every row of K sums to zero (sum_j grad N_j = 0),
    at the full 200x200 benchmark size; the assembled upper part is symmetric by construction."""
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    mesh = structured_quad_mesh(200, 200, "bilinear")
    pb = T.Problem2D.from_mesh(mesh)
    pb.set_model(T.Model2D(influence="fast_polynomial", radius=(0.05, 0.05), local_weight=0.5))
    r, pairs = pb.find_neighbours()
    assert r[0] == pytest.approx(0.05 + 0.005 * np.sqrt(2), rel=1e-12)
    off, _ = pb.neighbours()
    counts = np.diff(off).reshape(200, 200)
    assert counts[100, 100] == 421          # lattice points with |d| <= 10 + sqrt(2)
    pb.conductivity_matrix("FULL")
    rp, col, val = pb.matrix("inner")
    n = pb.n_nodes
    # no boundary conditions: a pure Neumann problem, copied out with the Lagrange
    # row and column (int N_i, which sum to the area); drop them
    assert rp.shape[0] == n + 2 and rp[-1] - rp[-2] == 1
    lagrange = col == n
    assert abs(val[lagrange].sum() - 1.0) < 1e-12
    rows = np.repeat(np.arange(n + 1), np.diff(rp))
    keep = ~lagrange
    rows, col, val = rows[keep], col[keep], val[keep]
    off_diag = col != rows
    sums = np.bincount(rows, weights=val, minlength=n) + np.bincount(col[off_diag], weights=val[off_diag], minlength=n)
    assert np.abs(sums).max() < 1e-12 * np.abs(val).max() * 50


@pytest.mark.parametrize("case", ["radiation", "convection", "neumann"])
def test_boundary_kinds_against_oracle_scaled(lib, case):
    """Convection, the radiation loop and pure Neumann problems on a 30 x 30 mesh,
    against the oracle (which solves the Neumann problem as the reference does, on
    the bordered system, and the radiation steps with Jacobi-preconditioned CG)."""
    import oracle
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    m = structured_quad_mesh(30, 30, "bilinear", jitter=0.1, seed=9)
    radius, p1 = 0.1, 0.5
    specs = {"radiation": [("left", dict(kind="temperature", value=300.0)),
                           ("right", dict(kind="combined", value=-50.0, heat_transfer=1.5, ambient_temperature=280.0,
                                          emissivity=0.4))],
             "convection": [("left", dict(kind="temperature", value=0.0)),
                            ("right", dict(kind="convection", heat_transfer=3.0, ambient_temperature=1.0))],
             "neumann": [("left", dict(kind="flux", value=-2.0)), ("right", dict(kind="flux", value=2.0))]}[case]
    energy = 0.25 if case == "neumann" else 0.0
    pb = T.Problem2D.from_mesh(m)
    pb.set_model(T.Model2D(influence="fast_polynomial", radius=(radius, radius), local_weight=p1, conductivity=(20.0,)))
    prob = oracle.Problem(2, m.nodes, m.elements)
    prob.set_model(influence=3, radius=(radius, radius), local_weight=p1, cond_kind=0, cond=(20.0, 0.0, 0.0))
    for group, d in specs:
        pb.add_boundary(T.Boundary(edges=m.boundaries[group], **d))
        if d["kind"] == "temperature":
            prob.add_boundary(0, m.boundaries[group], d["value"])
        else:
            prob.add_flux_boundary(gc.BOUNDARY_KINDS[d["kind"]], m.boundaries[group], d.get("value", 0.0),
                                   d.get("heat_transfer", 0.0), d.get("ambient_temperature", 0.0),
                                   d.get("emissivity", 0.0))
    pb.set_stationary_parameters(energy=energy)
    prob.set_stationary(energy=energy)
    pb.find_neighbours()
    prob.find_neighbours()
    prob.assemble(); prob.assemble_local(); prob.solve(tol=1e-14, maxit=50000)
    # each linear solve to 1e-12: the later radiation steps' right-hand sides are
    # small, and their relative residual floors near 1e-16 cond(K)
    t, rep = pb.stationary(tolerance=1e-12, max_iterations=50000)
    assert rel(t, prob.get("solution")) < SOLUTION_RTOL
    assert rep.neumann == (1 if case == "neumann" else 0)
    if case == "radiation":
        assert rep.nonlinear_iterations == int(prob.scalar("nonlinear_iterations")) >= 3
        tm, rep_m = pb.stationary(tolerance=1e-12, max_iterations=50000, precision="mixed")
        assert rel(tm, prob.get("solution")) < SOLUTION_RTOL and rep_m.nonlinear_iterations == rep.nonlinear_iterations
    if case == "neumann":
        assert abs(gc.lagrange_column({"elements": m.elements, "nodes": m.nodes, "jacobians": pb.quadrature()[1],
                                       "basis_qN": pb.basis()["basis_qN"],
                                       "basis_weights": pb.basis()["basis_weights"]}) @ t - energy) < 1e-12


def test_boundary_kind_errors(lib):
    """A convection edge that shares a node with a temperature group is rejected
    (the reference couples them through inserted Dirichlet entries); an unbalanced
    pure Neumann problem is rejected as the reference rejects it."""
    from nonlocal_gb300 import _lib
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    m = structured_quad_mesh(6, 6, "bilinear")
    pb = T.Problem2D.from_mesh(m)
    pb.set_model(T.Model2D(local_weight=1.0))
    pb.add_boundary(T.Boundary(edges=m.boundaries["left"], kind="temperature", value=0.0))
    pb.add_boundary(T.Boundary(edges=m.boundaries["down"], kind="convection", heat_transfer=1.0, ambient_temperature=1.0))
    with pytest.raises(_lib.NlgpuError, match="temperature boundary"):
        pb.stationary()
    pb.clear_boundaries()
    pb.add_boundary(T.Boundary(edges=m.boundaries["left"], kind="flux", value=1.0))
    pb.add_boundary(T.Boundary(edges=m.boundaries["right"], kind="flux", value=1.0))
    with pytest.raises(_lib.NlgpuError, match="unsolvable Neumann"):
        pb.stationary()
