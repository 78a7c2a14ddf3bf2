"""Node renumbering on the CUDA path (through the C ABI).

* nlgpu_cuthill_mckee against the reference's own permutations
  (mesh::utils::cuthill_mckee, stored in every fixture), bit-exact, for the
  local and the nonlocal node graph, plain and reverse;
* the reference's renumbered solve: SU2 file -> reader -> neighbours ->
  Cuthill-McKee -> nlgpu_renumbering -> assembly and solve must reproduce the
  reference's renumbered matrices (patterns bit-exact, values 1e-12) and
  temperature (1e-10);
* larger shuffled meshes against the oracle (including a window of node
  numbers too wide for shared memory), and renumbering invariance of the
  solution.
"""
import numpy as np
import pytest

import golden_cases as gc
from test_gpu_parity import MATRIX_RTOL, SOLUTION_RTOL, assert_csr_equal, gpu_problem, lib, rel  # noqa: F401

pytestmark = pytest.mark.gpu


def model_of(fx):
    from nonlocal_gb300 import thermal as T
    m = gc.model(fx["config"])
    return T.Model2D(influence={v: k for k, v in gc.INFLUENCE.items()}[m["influence"]], radius=m["radius"],
                     local_weight=m["local_weight"], n=m["n"], p=m["p"], q=m["q"],
                     conductivity=m["cond"][:m["cond_kind"] + 1])


@pytest.mark.parametrize("name", gc.STATIONARY_2D + ["b10_field_nonsym"])
def test_cuthill_mckee_matches_reference(lib, name, tmp_path):
    from nonlocal_gb300 import thermal as T
    fx = gc.load(name)
    pb = T.Problem2D.from_su2(gc.write_su2_text(fx, str(tmp_path / "mesh.su2")))
    pb.set_model(model_of(fx))
    if fx["config"].get("local_weight", 1) < 0.999:
        pb.find_neighbours(fx["config"].get("strategy", "MAX"))
    for key in [k for k in gc.CUTHILL_MCKEE if k in fx]:
        assert np.array_equal(pb.cuthill_mckee(*gc.CUTHILL_MCKEE[key]), fx[key]), key


@pytest.mark.parametrize("name", ["b12_shuffled_cm", "s5_shuffled_cm"])
def test_renumbered_solve_matches_reference(lib, name, tmp_path):
    from nonlocal_gb300 import thermal as T
    fx = gc.load(name)
    cfg = fx["config"]
    pb = T.Problem2D.from_su2(gc.write_su2_text(fx, str(tmp_path / "mesh.su2")))
    pb.set_model(model_of(fx))
    pb.find_neighbours(cfg.get("strategy", "MAX"))
    perm = pb.cuthill_mckee(*gc.CUTHILL_MCKEE["cm_" + cfg["renumber"]])
    assert np.array_equal(perm, fx["cm_" + cfg["renumber"]])
    pb.renumbering(perm)
    assert np.array_equal(pb.nodes, fx["nodes"]) and np.array_equal(pb.elements, fx["elements"])
    for key, spec in cfg.items():
        if key.startswith("bc."):
            kind, value = spec.split(":")
            edges = pb.su2.boundary(key[3:])   # the file's marker, renumbered with the mesh
            assert np.array_equal(edges, fx["bnd_" + key[3:]])
            pb.add_boundary(T.Boundary(edges=edges, kind=kind, value=float(value)))
    off, lst = pb.neighbours()
    assert np.array_equal(off, fx["neigh_offsets"]) and np.array_equal(lst, fx["neigh_list"])
    pb.conductivity_matrix("FULL")
    assert_csr_equal(pb.matrix("inner"), fx, "K_inner")
    assert_csr_equal(pb.matrix("bound"), fx, "K_bound")
    t, _ = pb.stationary(tolerance=1e-14)
    assert rel(t, fx["temperature"]) < SOLUTION_RTOL


def shuffled_problem(nx, element, radius, local_weight, seed):
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    m = structured_quad_mesh(nx, nx, element, jitter=0.1, seed=seed, shuffle_seed=seed + 1)
    pb = T.Problem2D.from_mesh(m)
    pb.set_model(T.Model2D(influence="fast_polynomial", radius=(radius, radius), local_weight=local_weight))
    return m, pb


def oracle_of(m, radius, local_weight):
    import oracle
    prob = oracle.Problem(2 if m.nodes_per_element == 4 else 3, m.nodes, m.elements)
    prob.set_model(influence=3, n=2, p=2, q=1.0, radius=(radius, radius), local_weight=local_weight,
                   cond_kind=0, cond=(1.0, 0.0, 0.0))
    if local_weight < 0.999:
        prob.find_neighbours()
    return prob


@pytest.mark.parametrize("nx,element,radius", [(40, "bilinear", 0.1), (16, "serendipity", 0.2)])
def test_cuthill_mckee_scaled_against_oracle(lib, nx, element, radius):
    m, pb = shuffled_problem(nx, element, radius, 0.5, seed=nx)
    prob = oracle_of(m, radius, 0.5)
    for only_local in (True, False):
        for reverse in (False, True):
            assert np.array_equal(pb.cuthill_mckee(only_local, reverse), prob.cuthill_mckee(only_local, reverse)), \
                (only_local, reverse)


def test_cuthill_mckee_wide_window(lib):
    """400 000 nodes numbered at random: a node's window of candidate numbers
    spans the whole mesh, wider than the shared-memory bitmap, so the graph
    kernels run on per-warp global bitmaps."""
    m, pb = shuffled_problem(632, "bilinear", 0.01, 1.0, seed=5)
    assert m.n_nodes > 12288 * 32
    prob = oracle_of(m, 0.01, 1.0)
    assert np.array_equal(pb.cuthill_mckee(True, False), prob.cuthill_mckee(True, False))


def test_renumbering_keeps_the_solution(lib):
    """The permuted system has the permuted solution: T_renumbered[perm] == T."""
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import relabel_nodes
    solutions = []
    perm = None
    for renumber in (False, True):
        m, pb = shuffled_problem(30, "bilinear", 0.12, 0.5, seed=3)
        if renumber:
            pb.find_neighbours()
            perm = pb.cuthill_mckee(False, False)
            pb.renumbering(perm)
            m = relabel_nodes(m, perm)
            assert np.array_equal(pb.nodes, m.nodes) and np.array_equal(pb.elements, m.elements)
        pb.add_boundary(T.Boundary(edges=m.boundaries["left"], kind="temperature", value=0.0))
        pb.add_boundary(T.Boundary(edges=m.boundaries["right"], kind="flux", value=1.0))
        t, rep = pb.stationary(tolerance=1e-12)
        solutions.append(t)
    assert rel(solutions[1][perm], solutions[0]) < 1e-9


def test_renumbering_rejects_bad_permutations(lib):
    from nonlocal_gb300 import _lib
    m, pb = shuffled_problem(6, "bilinear", 0.3, 1.0, seed=1)
    bad = np.arange(m.n_nodes)
    bad[3] = bad[4]
    with pytest.raises(_lib.NlgpuError, match="same"):
        pb.renumbering(bad)
    with pytest.raises(_lib.NlgpuError, match="range"):
        pb.renumbering(np.arange(m.n_nodes) + 1)


def test_disconnected_graph_is_rejected(lib):
    from nonlocal_gb300 import _lib
    from nonlocal_gb300 import thermal as T
    nodes = np.array([[0, 0], [1, 0], [1, 1], [0, 1], [3, 0], [4, 0], [4, 1], [3, 1]], dtype=float)
    elements = np.array([[0, 1, 2, 3], [4, 5, 6, 7]])
    pb = T.Problem2D("bilinear", nodes, elements)
    pb.set_model(T.Model2D(local_weight=1.0))
    with pytest.raises(_lib.NlgpuError, match="not connected"):
        pb.cuthill_mckee(True, False)
