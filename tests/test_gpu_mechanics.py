"""Nonlocal plane elasticity (DoF = 2) on the GPU against the reference's own
runs of equilibrium_equation (tests/golden/m8_mechanical: nonlocal bilinear,
clamped left side, pressure on the right; s4_mechanical_local: local jittered
serendipity, clamped bottom, pressure on the top): stiffness patterns
bit-exact, values and right-hand sides within 1e-12 (max-norm scaled),
displacement within 1e-10 relative L2 -- and, at a larger size, the property
every stiffness matrix has: rigid translations produce no force."""
import numpy as np
import pytest

import golden_cases as gc

pytestmark = pytest.mark.gpu

MATRIX_RTOL = 1e-12
SOLUTION_RTOL = 1e-10
CASES = ["m8_mechanical", "s4_mechanical_local"]


@pytest.fixture(scope="module")
def lib():
    from nonlocal_gb300 import _lib, build
    build.build()
    _lib.load()
    if _lib.device_count() == 0:
        pytest.fail("no CUDA device visible to the nlgpu library")
    return _lib


def mechanical_conditions(fx):
    """mbc.<group> = <x>,<y>, each d:<value> (displacement) or p:<value> (pressure)."""
    from nonlocal_gb300 import thermal as T
    out = []
    for key, spec in fx["config"].items():
        if not key.startswith("mbc."):
            continue
        comps = []
        for part in spec.split(","):
            comps.append(("displacement" if part[0] == "d" else "pressure", float(part[2:])))
        out.append(T.MechanicalBoundary(edges=fx["bnd_" + key[4:]], x=comps[0], y=comps[1]))
    return out


def gpu_problem(fx):
    from nonlocal_gb300 import thermal as T
    cfg = fx["config"]
    pb = T.MechanicalProblem2D(gc.element_type(fx), fx["nodes"], fx["elements"])
    m = gc.model(cfg)
    pb.set_model(T.Model2D(influence={v: k for k, v in gc.INFLUENCE.items()}[m["influence"]], radius=m["radius"],
                           local_weight=m["local_weight"], n=m["n"], p=m["p"], q=m["q"]))
    pb.set_elastic(T.ElasticParameters("isotropic", (float(cfg.get("young_modulus", 210.0)),),
                                       (float(cfg.get("poissons_ratio", 0.3)),)))
    for b in mechanical_conditions(fx):
        pb.add_mechanical_boundary(b)
    if m["local_weight"] < 0.999:
        pb.find_neighbours()
    return pb


def assert_csr(got, fx, name):
    rp, col, val = got
    assert np.array_equal(rp, fx[name + "_rowptr"]), f"{name}: row pointers"
    assert np.array_equal(col, fx[name + "_col"]), f"{name}: columns"
    ref = fx[name + "_val"]
    scale = np.abs(ref).max() if ref.size else 1.0
    np.testing.assert_allclose(val, ref, rtol=MATRIX_RTOL, atol=MATRIX_RTOL * scale, err_msg=name)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("name", CASES)
def test_stiffness_matrices_and_rhs(lib, name):
    fx = gc.load(name)
    pb = gpu_problem(fx)
    if fx["config"].get("local_weight", 1) < 0.999:
        off, lst = pb.neighbours()
        assert np.array_equal(off, fx["neigh_offsets"]) and np.array_equal(lst, fx["neigh_list"])
    pb.stiffness_matrix("FULL")
    assert_csr(pb.stiffness("inner"), fx, "K_inner")
    assert_csr(pb.stiffness("bound"), fx, "K_bound")
    f, f0 = pb.mechanical_rhs()
    scale = np.abs(fx["rhs"]).max()
    np.testing.assert_allclose(f0, fx["rhs_init"], rtol=MATRIX_RTOL, atol=MATRIX_RTOL * scale)
    np.testing.assert_allclose(f, fx["rhs"], rtol=MATRIX_RTOL, atol=MATRIX_RTOL * scale)
    pb.stiffness_matrix("LOCAL")
    assert_csr(pb.stiffness("local"), fx, "K_local")


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_displacement(lib, name, precision):
    """equilibrium_equation's displacement (ILLT-CG for the nonlocal case, CG for
    the local one, as the reference's defaults), FP64 or mixed precision."""
    fx = gc.load(name)
    pb = gpu_problem(fx)
    u, rep = pb.equilibrium(tolerance=1e-13, max_iterations=20000, precision=precision)
    assert rep.residual <= 1e-13
    assert rel(u.reshape(-1), fx["displacement"]) < SOLUTION_RTOL
    clamped = np.flatnonzero(fx["is_inner"] == 0)
    assert np.all(u.reshape(-1)[clamped] == 0.0)


def test_rigid_translations_produce_no_force(lib):
    """Without displacement conditions every row of the nonlocal stiffness sums
    to zero per component (sum_j grad N_j = 0): K applied to a unit translation
    in x or y vanishes to rounding, here on a 48x48 jittered serendipity mesh."""
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    mesh = structured_quad_mesh(48, 48, "serendipity", jitter=0.2, seed=3)
    pb = T.MechanicalProblem2D.from_mesh(mesh)
    pb.set_model(T.Model2D(influence="exponential", radius=(0.06, 0.06), local_weight=0.3))
    h = pb.set_elastic(T.ElasticParameters("anisotropic", (200.0, 120.0), (0.25, 0.15), 60.0, 0.4))
    assert h[4] != 0.0 and h[5] != 0.0
    pb.add_mechanical_boundary(T.MechanicalBoundary(edges=mesh.boundaries["up"], x=("pressure", 1.0)))
    pb.find_neighbours()
    pb.stiffness_matrix("FULL")
    rp, col, val = pb.stiffness("inner")
    n2 = 2 * pb.n_nodes
    rows = np.repeat(np.arange(n2), np.diff(rp))
    for comp in (0, 1):
        t = np.zeros(n2)
        t[comp::2] = 1.0
        # symmetric product from the upper storage
        y = np.bincount(rows, weights=val * t[col], minlength=n2)
        off = col != rows
        y += np.bincount(col[off], weights=val[off] * t[rows[off]], minlength=n2)
        assert np.abs(y).max() <= 1e-11 * np.abs(val).max() * np.sqrt(np.diff(rp).max()), comp
