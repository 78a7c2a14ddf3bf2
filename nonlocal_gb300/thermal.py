"""Host-side mirror of NonLocFEM's thermal solver API over the nlgpu C ABI.

Names and argument meaning follow the reference:

* ``Problem2D`` holds what the reference spreads over ``mesh::mesh_2d``,
  ``parameters_2d`` and ``thermal_boundaries_conditions_2d``: one device
  context (``nlgpu_ctx``) per problem;
* ``find_neighbours`` -- ``mesh::find_neighbours`` (find_neighbours.hpp:120-160);
* ``Problem2D.conductivity_matrix`` -- ``conductivity_matrix_2d::compute``
  (conductivity_matrix_2d.hpp:166-193);
* ``stationary_heat_equation_solver_2d`` (stationary_heat_equation_solver_2d.hpp:46-120);
* ``NonstationaryHeatEquationSolver2D`` (nonstationary_heat_equation_solver_2d.hpp:16-106);
* ``conjugate_gradient`` -- ``slae::conjugate_gradient`` with the ILLT
  preconditioner (conjugate_gradient.hpp:15-79, eigen_preconditioner.hpp:57);
* ``stationary_heat_equation_solver_1d`` (stationary_heat_equation_solver_1d.hpp:43-122);
* ``equilibrium_equation`` / ``MechanicalProblem2D`` -- nonlocal plane elasticity
  (mechanical/equilibrium_equation_2d.hpp:19-60, stiffness_matrix_2d.hpp).

Errors raise ``NlgpuError`` (the reference throws std::domain_error /
std::logic_error); every compute call runs on the GPU.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L
from .meshgen import BILINEAR, SERENDIPITY, QuadMesh

ELEMENT_TYPE = {BILINEAR: L.BILINEAR, SERENDIPITY: L.QUADRATIC_SERENDIPITY}


@dataclass
class Model2D:
    """model_parameters<2, T> with its influence function and constant conductivity."""

    influence: str = "fast_polynomial"      # constant | polynomial | exponential | fast_polynomial
    radius: tuple[float, float] = (0.1, 0.1)
    local_weight: float = 1.0               # p1
    n: int = 2                              # powered-distance exponent
    p: int = 2
    q: float | None = None                  # default 1 (polynomial) / 0.5 (exponential)
    conductivity: tuple[float, ...] = (1.0,)  # (l,) | (lx, ly) | (xx, yy, xy)

    def to_c(self) -> L.Model2D:
        m = L.Model2D()
        m.influence = L.INFLUENCE[self.influence]
        m.n, m.p = int(self.n), int(self.p)
        m.q = float(self.q if self.q is not None else (0.5 if self.influence == "exponential" else 1.0))
        m.radius[0], m.radius[1] = float(self.radius[0]), float(self.radius[1])
        m.local_weight = float(self.local_weight)
        c = tuple(float(v) for v in self.conductivity)
        m.conductivity_kind = L.CONDUCTIVITY_KIND[len(c)]
        for k, v in enumerate(c):
            m.conductivity[k] = v
        return m


@dataclass
class Boundary:
    """A boundary group (thermal_boundary_conditions_2d.hpp:9-98).

    ``kind``: 'temperature' (``value``, or per-node ``node_values``), 'flux'
    (``value``), 'convection' (``heat_transfer``, ``ambient_temperature``),
    'radiation' (``emissivity``) or 'combined' (flux ``value`` and all three)."""

    edges: np.ndarray
    kind: str = "temperature"
    value: float = 0.0
    node_values: np.ndarray | None = None
    heat_transfer: float = 0.0
    ambient_temperature: float = 0.0
    emissivity: float = 0.0


BOUNDARY_KIND = {"temperature": L.BC_TEMPERATURE, "flux": L.BC_FLUX, "convection": L.BC_CONVECTION,
                 "radiation": L.BC_RADIATION, "combined": L.BC_COMBINED_FLUX}


@dataclass
class SolveReport:
    values: dict = field(default_factory=dict)

    def __getattr__(self, name):
        try:
            return self.values[name]
        except KeyError as e:
            raise AttributeError(name) from e


@dataclass
class Su2Mesh:
    """An SU2 file as the reference's mesh_container_2d numbers it.

    ``element`` is "bilinear" / "serendipity" when all 2D elements have that
    type (else None); ``groups`` maps each marker (and "DEFAULT", the 2D
    elements in no 2D marker) to (dimension, elements [count][nodes], first
    index in the container), in the container's group order."""

    element: str | None
    nodes: np.ndarray
    elements: np.ndarray
    groups: dict[str, tuple[int, np.ndarray, int]]

    def boundary(self, name: str) -> np.ndarray:
        dim, edges, _ = self.groups[name]
        if dim != 1:
            raise ValueError(f"group {name!r} is not a boundary group")
        return edges

    def renumbered(self, p: np.ndarray) -> "Su2Mesh":
        nodes = np.empty_like(self.nodes)
        nodes[p] = self.nodes
        return Su2Mesh(self.element, nodes, p[self.elements],
                       {k: (d, p[e], f) for k, (d, e, f) in self.groups.items()})


def read_su2(path: str) -> Su2Mesh:
    """mesh_parser<T, I, mesh_format::SU2>::parse (su2_parser.hpp:165-195) through
    nlgpu_su2_read: host code, no GPU needed."""
    lib = L.load()
    h = ctypes.c_void_p()
    st = lib.nlgpu_su2_read(str(path).encode(), ctypes.byref(h))
    if st != L.OK:
        raise L.NlgpuError(st, lib.nlgpu_su2_last_error().decode())
    try:
        n, e2 = ctypes.c_int64(), ctypes.c_int64()
        nen, et, ng = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        L.check(lib.nlgpu_su2_info(h, ctypes.byref(n), ctypes.byref(e2), ctypes.byref(nen), ctypes.byref(et),
                                   ctypes.byref(ng)))
        nodes = np.empty((n.value, 2))
        L.check(lib.nlgpu_su2_nodes(h, L.ptr(nodes)))
        elements = np.empty((e2.value, max(nen.value, 1)), dtype=np.int64)
        if nen.value:
            L.check(lib.nlgpu_su2_elements_2d(h, L.ptr(elements)))
        groups = {}
        name = ctypes.create_string_buffer(4096)
        for g in range(ng.value):
            dim, gnen = ctypes.c_int(), ctypes.c_int()
            first, count = ctypes.c_int64(), ctypes.c_int64()
            L.check(lib.nlgpu_su2_group(h, g, name, len(name), ctypes.byref(dim), ctypes.byref(first),
                                        ctypes.byref(count), ctypes.byref(gnen), None))
            members = np.empty((count.value, gnen.value), dtype=np.int64)
            L.check(lib.nlgpu_su2_group(h, g, None, 0, None, None, None, None, L.ptr(members)))
            groups[name.value.decode()] = (dim.value, members, first.value)
    finally:
        lib.nlgpu_su2_free(h)
    element = {L.BILINEAR: BILINEAR, L.QUADRATIC_SERENDIPITY: SERENDIPITY}.get(et.value)
    return Su2Mesh(element, nodes, elements, groups)


def cuthill_mckee(problem: "Problem2D", only_local: bool = False, reverse: bool = False) -> np.ndarray:
    """mesh::utils::cuthill_mckee(mesh, only_local, reverse) (cuthill_mckee.hpp:166-171)."""
    return problem.cuthill_mckee(only_local, reverse)


class Context:
    """An nlgpu_ctx: device state of one problem on one CUDA stream."""

    def __init__(self, stream: int | None = None):
        self._lib = L.load()
        self._h = ctypes.c_void_p()
        L.check(self._lib.nlgpu_create(ctypes.byref(self._h), stream))

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.nlgpu_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def synchronize(self) -> None:
        L.check(self._lib.nlgpu_synchronize(self._h))


class Problem2D(Context):
    """One 2D thermal problem held on the GPU."""

    def __init__(self, element: str | int, nodes, elements, stream: int | None = None):
        super().__init__(stream)
        et = ELEMENT_TYPE.get(element, element)
        self.nodes = L.f64(nodes)
        self.elements = L.i64(elements)
        L.check(self._lib.nlgpu_mesh_2d(self._h, int(et), self.nodes.shape[0], L.ptr(self.nodes),
                                        self.elements.shape[0], L.ptr(self.elements)))
        self.n_nodes = int(self.nodes.shape[0])
        self.n_elements = int(self.elements.shape[0])
        self.nodes_per_element = int(self.elements.shape[1])
        self.qnodes = 4 if self.nodes_per_element == 4 else 9

    @classmethod
    def from_mesh(cls, mesh: QuadMesh, **kw) -> "Problem2D":
        return cls(mesh.element, mesh.nodes, mesh.elements, **kw)

    @classmethod
    def from_su2(cls, path: str, **kw) -> "Problem2D":
        """mesh_2d(path): the mesh of an SU2 file in the reference's element
        numbering; the file's markers are kept in ``self.su2`` (see ``read_su2``)."""
        m = read_su2(path)
        if m.element is None:
            raise L.NlgpuError(3, "the 2D elements are not all bilinear or all 8-node serendipity")
        p = cls(m.element, m.nodes, m.elements, **kw)
        p.su2 = m
        return p

    # ---- renumbering ------------------------------------------------------------
    def cuthill_mckee(self, only_local: bool = False, reverse: bool = False) -> np.ndarray:
        """mesh::utils::cuthill_mckee: permutation[old] = new (the inverse with reverse=True)."""
        perm = np.empty(self.n_nodes, dtype=np.int64)
        L.check(self._lib.nlgpu_cuthill_mckee(self._h, int(only_local), int(reverse), L.ptr(perm)))
        return perm

    def renumbering(self, permutation) -> None:
        """mesh_2d::renumbering: node i becomes node permutation[i]."""
        p = L.i64(permutation)
        if p.shape != (self.n_nodes,):
            raise ValueError(f"the permutation needs {self.n_nodes} entries")
        L.check(self._lib.nlgpu_renumbering(self._h, L.ptr(p)))
        nodes = np.empty_like(self.nodes)
        nodes[p] = self.nodes
        self.nodes, self.elements = nodes, p[self.elements]
        if getattr(self, "su2", None) is not None:
            self.su2 = self.su2.renumbered(p)

    # ---- model, boundaries ------------------------------------------------
    def set_model(self, model: Model2D) -> None:
        m = model.to_c()
        L.check(self._lib.nlgpu_set_model_2d(self._h, ctypes.byref(m)))
        self.model = model

    def set_conductivity_field(self, values: np.ndarray | None) -> None:
        self._cond = None if values is None else L.f64(values).reshape(-1)
        L.check(self._lib.nlgpu_set_conductivity_field(self._h, L.ptr(self._cond)))

    def set_capacity(self, capacity: float = 1.0, density: float = 1.0) -> None:
        L.check(self._lib.nlgpu_set_capacity(self._h, capacity, density))

    def add_boundary(self, b: Boundary) -> None:
        edges = L.i64(b.edges)
        kind = BOUNDARY_KIND[b.kind]
        if kind == L.BC_TEMPERATURE:
            nv = None if b.node_values is None else L.f64(b.node_values)
            L.check(self._lib.nlgpu_add_boundary_2d(self._h, kind, edges.shape[0], edges.shape[1], L.ptr(edges),
                                                    float(b.value), L.ptr(nv)))
        else:
            L.check(self._lib.nlgpu_add_flux_boundary_2d(self._h, kind, edges.shape[0], edges.shape[1], L.ptr(edges),
                                                         float(b.value), float(b.heat_transfer),
                                                         float(b.ambient_temperature), float(b.emissivity)))

    def set_stationary_parameters(self, tolerance: float = 1e-8, max_iterations: int = 100, energy: float = 0.0,
                                  initial_temperature=None) -> None:
        """stationary_equation_parameters_2d: the radiation loop's stop test, int T of a
        pure Neumann problem, and the loop's initial temperature."""
        self._t0 = None if initial_temperature is None else L.f64(initial_temperature)
        L.check(self._lib.nlgpu_set_stationary_parameters(self._h, float(tolerance), int(max_iterations),
                                                          float(energy), L.ptr(self._t0)))

    def system_rows(self) -> int:
        """n_nodes, or n_nodes + 1 for a pure Neumann problem (the Lagrange row)."""
        rows = ctypes.c_int64()
        L.check(self._lib.nlgpu_get_system_rows(self._h, ctypes.byref(rows)))
        return int(rows.value)

    def clear_boundaries(self) -> None:
        L.check(self._lib.nlgpu_clear_boundaries(self._h))

    def set_source(self, value: float = 0.0, per_qnode: np.ndarray | None = None) -> None:
        self._src = None if per_qnode is None else L.f64(per_qnode).reshape(-1)
        L.check(self._lib.nlgpu_set_source(self._h, float(value), L.ptr(self._src)))

    def set_dirichlet_values(self, values: np.ndarray | None) -> None:
        self._dv = None if values is None else L.f64(values)
        L.check(self._lib.nlgpu_set_dirichlet_values(self._h, L.ptr(self._dv)))

    # ---- mesh data ------------------------------------------------------------
    def quadrature(self):
        E, nq, nen = self.n_elements, self.qnodes, self.nodes_per_element
        qc, jac, der = np.empty((E, nq, 2)), np.empty((E, nq)), np.empty((E, nen, nq, 2))
        L.check(self._lib.nlgpu_get_quadrature(self._h, L.ptr(qc), L.ptr(jac), L.ptr(der)))
        return qc, jac, der

    def basis(self) -> dict:
        nen, nq = ctypes.c_int(), ctypes.c_int()
        L.check(self._lib.nlgpu_get_basis(self._h, ctypes.byref(nen), ctypes.byref(nq), None, None, None, None, None))
        qN, qNxi, qNeta = (np.empty(nen.value * nq.value) for _ in range(3))
        w, c = np.empty(nq.value), np.empty(nen.value)
        L.check(self._lib.nlgpu_get_basis(self._h, None, None, L.ptr(qN), L.ptr(qNxi), L.ptr(qNeta), L.ptr(w), L.ptr(c)))
        return {"basis_qN": qN, "basis_qNxi": qNxi, "basis_qNeta": qNeta, "basis_weights": w, "basis_centre": c}

    def set_assembly_precision(self, kind: str = "auto") -> None:
        """How the nonlocal pair blocks are computed: "auto" (float-float on the FP32
        pipes for mixed-precision solves, FP64 otherwise), "ff" or "fp64" always."""
        L.check(self._lib.nlgpu_set_option(self._h, L.OPTION_ASSEMBLY_PRECISION, L.ASSEMBLY[kind]))

    def set_assembly_warps(self, warps: int = 0) -> None:
        """Warps per CTA of the float-float pair assembly: 16 or 32, or 0 to time
        both on a sample of elements at the first float-float assembly and keep
        the faster."""
        L.check(self._lib.nlgpu_set_option(self._h, L.OPTION_ASSEMBLY_WARPS, int(warps)))

    def assembly_tuning(self) -> dict:
        """Warps per CTA of the last float-float assembly and the last tuning's
        sample times (ms) with 16 and 32 warps."""
        w = ctypes.c_int()
        ms = (ctypes.c_double * 2)()
        L.check(self._lib.nlgpu_assembly_tuning(self._h, ctypes.byref(w), ms))
        return {"warps": w.value, "sample_ms_16": ms[0], "sample_ms_32": ms[1]}

    # ---- neighbours -----------------------------------------------------------
    def find_neighbours(self, strategy: str = "MAX") -> tuple[np.ndarray, int]:
        r = np.empty(2)
        pairs = ctypes.c_int64()
        L.check(self._lib.nlgpu_find_neighbours(self._h, L.EXPAND[strategy], L.ptr(r), ctypes.byref(pairs)))
        self.pairs = int(pairs.value)
        return r, self.pairs

    def neighbours(self) -> tuple[np.ndarray, np.ndarray]:
        off = np.empty(self.n_elements + 1, dtype=np.int64)
        L.check(self._lib.nlgpu_get_neighbours(self._h, L.ptr(off), None))
        lst = np.empty(int(off[-1]), dtype=np.int64)
        L.check(self._lib.nlgpu_get_neighbours(self._h, None, L.ptr(lst)))
        return off, lst

    # ---- assembly -------------------------------------------------------------
    def conductivity_matrix(self, part: str = "FULL") -> tuple[int, int]:
        ni, nb = ctypes.c_int64(), ctypes.c_int64()
        L.check(self._lib.nlgpu_conductivity_matrix_2d(self._h, L.PART_FULL if part == "FULL" else L.PART_LOCAL,
                                                       ctypes.byref(ni), ctypes.byref(nb)))
        self._nnz = {"FULL": (int(ni.value), int(nb.value))} if part == "FULL" else {"LOCAL": (int(ni.value), 0)}
        if part == "FULL":
            self.nnz_inner, self.nnz_bound = int(ni.value), int(nb.value)
        else:
            self.nnz_local = int(ni.value)
        return int(ni.value), int(nb.value)

    def matrix(self, which: str = "inner") -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        code = {"inner": L.MATRIX_INNER, "bound": L.MATRIX_BOUND, "local": L.MATRIX_LOCAL}[which]
        try:   # a pure Neumann problem's matrices carry the Lagrange row and column
            rows = self.system_rows()
        except L.NlgpuError:
            rows = self.n_nodes   # only the LOCAL part assembled
        rp = np.empty(rows + 1, dtype=np.int64)
        L.check(self._lib.nlgpu_get_matrix(self._h, code, L.ptr(rp), None, None))
        col = np.empty(int(rp[-1]), dtype=np.int64)
        val = np.empty(int(rp[-1]))
        L.check(self._lib.nlgpu_get_matrix(self._h, code, None, L.ptr(col), L.ptr(val)))
        return rp, col, val

    def rhs(self) -> tuple[np.ndarray, np.ndarray]:
        rows = self.system_rows()
        f, f0 = np.empty(rows), np.empty(rows)
        L.check(self._lib.nlgpu_get_rhs(self._h, L.ptr(f), L.ptr(f0)))
        return f, f0

    def calc_flux(self, temperature) -> tuple[np.ndarray, np.ndarray]:
        """heat_equation_solution_2d::calc_flux: the nodal heat flux (x, y) of a
        temperature field on this problem's mesh and model."""
        t = L.f64(temperature)
        if t.shape != (self.n_nodes,):
            raise ValueError(f"temperature needs {self.n_nodes} nodal values")
        fx, fy = np.empty(self.n_nodes), np.empty(self.n_nodes)
        L.check(self._lib.nlgpu_calc_flux(self._h, L.ptr(t), L.ptr(fx), L.ptr(fy)))
        return fx, fy

    # ---- solves -----------------------------------------------------------------
    @staticmethod
    def _options(tolerance, max_iterations, preconditioner, precision, inner_tolerance=0.0,
                 triangular_sweeps=0, coarse_aggregates=0, coarse_aspect=0.0) -> L.SolveOptions:
        o = L.SolveOptions()
        o.tolerance, o.max_iterations = float(tolerance), int(max_iterations)
        o.preconditioner, o.precision = L.PRECONDITIONER[preconditioner], L.PRECISION[precision]
        o.inner_tolerance = float(inner_tolerance)
        o.triangular_sweeps = int(triangular_sweeps)
        o.coarse_aggregates = int(coarse_aggregates)
        o.coarse_aspect = float(coarse_aspect)
        return o

    def stationary(self, tolerance=1e-10, max_iterations=10000, preconditioner="illt", precision="fp64",
                   check_convergence=True, inner_tolerance=0.0, triangular_sweeps=0, coarse_aggregates=0,
                   coarse_aspect=0.0):
        """stationary_heat_equation_solver_2d; precision "mixed" runs the FP32 inner
        solve with FP64 refinement (inner_tolerance: reduction per inner solve;
        triangular_sweeps: Jacobi sweeps per triangle of the FP32 ILLT application,
        0 the default, -1 exact level-scheduled substitution; coarse_aggregates > 0
        adds a coarse-space correction over about that many node aggregates, whose
        grid cells are coarse_aspect times wider than high (0: from the
        conductivity))."""
        o = self._options(tolerance, max_iterations, preconditioner, precision, inner_tolerance, triangular_sweeps,
                          coarse_aggregates, coarse_aspect)
        t = np.empty(self.n_nodes)
        rep = L.SolveReport()
        rc = self._lib.nlgpu_stationary_2d(self._h, ctypes.byref(o), L.ptr(t), ctypes.byref(rep))
        if rc != L.OK and (check_convergence or rc != 6):
            L.check(rc)
        return t, SolveReport(rep.as_dict())

    def solve_assembled(self, tolerance=1e-10, max_iterations=10000, preconditioner="illt", precision="fp64",
                        inner_tolerance=0.0, triangular_sweeps=0):
        o = self._options(tolerance, max_iterations, preconditioner, precision, inner_tolerance, triangular_sweeps)
        t = np.empty(self.n_nodes)
        rep = L.SolveReport()
        L.check(self._lib.nlgpu_solve_assembled(self._h, ctypes.byref(o), L.ptr(t), ctypes.byref(rep)))
        return t, SolveReport(rep.as_dict())

    # ---- learned correction on top of ILLT ------------------------------------------
    def train_learned_preconditioner(self, right_hand_sides=4, epochs=20, batch=8, learning_rate=1e-3,
                                     seed=0) -> dict:
        """Harvests (r, e) pairs from plain ILLT-CG on this (assembled) system and
        trains the message-passing correction on the GPU; returns the report."""
        o = L.TrainOptions(int(right_hand_sides), int(epochs), int(batch), float(learning_rate), int(seed))
        rep = L.TrainReport()
        L.check(self._lib.nlgpu_mpnn_train(self._h, ctypes.byref(o), ctypes.byref(rep)))
        return rep.as_dict()

    def learned_weights(self) -> np.ndarray:
        w = np.empty(L.MPNN_PARAMS, dtype=np.float32)
        L.check(self._lib.nlgpu_mpnn_get_weights(self._h, w.ctypes.data))
        return w

    def set_learned_weights(self, w, enabled: bool = True) -> None:
        """Weights of the learned correction (and the validation gate's decision)."""
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == L.MPNN_PARAMS
        L.check(self._lib.nlgpu_mpnn_set_weights(self._h, w.ctypes.data))
        L.check(self._lib.nlgpu_mpnn_set_enabled(self._h, int(bool(enabled))))

    def learned_loss_grad(self, r, e):
        """One (r, e) pair on the assembled system: z = ILLT^-1 r, P(r), loss, gradient."""
        r = np.ascontiguousarray(r, dtype=np.float32)
        e = np.ascontiguousarray(e, dtype=np.float32)
        z = np.empty_like(r)
        p = np.empty_like(r)
        g = np.empty(L.MPNN_PARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        L.check(self._lib.nlgpu_mpnn_loss_grad(self._h, r.ctypes.data, e.ctypes.data, z.ctypes.data, p.ctypes.data,
                                               ctypes.byref(loss), g.ctypes.data))
        return z, p, loss.value, g


@dataclass
class ElasticParameters:
    """elastic_parameters_t (elastic_parameters.hpp): constant isotropic (E, nu),
    orthotropic (E_x, E_y, nu_x, nu_y, G) or anisotropic (the orthotropic ones
    and a rotation angle)."""

    kind: str = "isotropic"
    young_modulus: tuple[float, ...] = (210.0,)
    poissons_ratio: tuple[float, ...] = (0.3,)
    shear_modulus: float = 210.0 / 13.0
    angle: float = 0.0

    def values(self) -> np.ndarray:
        if self.kind == "isotropic":
            return np.array([self.young_modulus[0], self.poissons_ratio[0]], dtype=np.float64)
        v = [*self.young_modulus[:2], *self.poissons_ratio[:2], self.shear_modulus]
        if self.kind == "anisotropic":
            v.append(self.angle)
        return np.array(v, dtype=np.float64)


@dataclass
class MechanicalBoundary:
    """mechanical_boundary_conditions_2d of one group: per component None,
    ("displacement", value) (displacement_2d) or ("pressure", value) (pressure_2d)."""

    edges: np.ndarray
    x: tuple | None = None
    y: tuple | None = None


class MechanicalProblem2D(Problem2D):
    """A plane-elasticity problem on the GPU (DoF = 2, rows 2 node + component):
    the mesh, neighbours and nonlocal model of Problem2D, Hooke parameters and
    displacement / pressure boundaries."""

    def set_elastic(self, parameters: ElasticParameters) -> np.ndarray:
        """Sets the Hooke matrix; returns h11, h12, h66, h22, h16, h26."""
        v = parameters.values()
        h = np.empty(6)
        L.check(self._lib.nlgpu_set_elastic_2d(self._h, L.ELASTIC[parameters.kind], L.ptr(v), L.ptr(h)))
        self.elastic = parameters
        return h

    def add_mechanical_boundary(self, b: MechanicalBoundary) -> None:
        edges = L.i64(b.edges)
        kx, vx = (None, 0.0) if b.x is None else b.x
        ky, vy = (None, 0.0) if b.y is None else b.y
        L.check(self._lib.nlgpu_add_mechanical_boundary_2d(self._h, edges.shape[0], edges.shape[1], L.ptr(edges),
                                                           L.MECH_CONDITION[kx], float(vx), L.MECH_CONDITION[ky],
                                                           float(vy)))

    def clear_mechanical_boundaries(self) -> None:
        L.check(self._lib.nlgpu_clear_mechanical_boundaries(self._h))

    def stiffness_matrix(self, part: str = "FULL") -> tuple[int, int]:
        """stiffness_matrix::compute of the FULL or LOCAL part."""
        ni, nb = ctypes.c_int64(), ctypes.c_int64()
        L.check(self._lib.nlgpu_stiffness_matrix_2d(self._h, L.PART_FULL if part == "FULL" else L.PART_LOCAL,
                                                    ctypes.byref(ni), ctypes.byref(nb)))
        return int(ni.value), int(nb.value)

    def stiffness(self, which: str = "inner") -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        code = {"inner": L.MATRIX_INNER, "bound": L.MATRIX_BOUND, "local": L.MATRIX_LOCAL}[which]
        rp = np.empty(2 * self.n_nodes + 1, dtype=np.int64)
        L.check(self._lib.nlgpu_get_stiffness_matrix(self._h, code, L.ptr(rp), None, None))
        col = np.empty(int(rp[-1]), dtype=np.int64)
        val = np.empty(int(rp[-1]))
        L.check(self._lib.nlgpu_get_stiffness_matrix(self._h, code, None, L.ptr(col), L.ptr(val)))
        return rp, col, val

    def mechanical_rhs(self) -> tuple[np.ndarray, np.ndarray]:
        f, f0 = np.empty(2 * self.n_nodes), np.empty(2 * self.n_nodes)
        L.check(self._lib.nlgpu_get_mechanical_rhs(self._h, L.ptr(f), L.ptr(f0)))
        return f, f0

    def equilibrium(self, tolerance=1e-10, max_iterations=10000, preconditioner=None, precision="fp64",
                    triangular_sweeps=0):
        """equilibrium_equation: assembly, boundary conditions and the CG solve
        (ILLT of the LOCAL stiffness for a nonlocal model, identity for a local
        one, unless `preconditioner` says otherwise).  Returns the displacement
        as [n][2] and the report."""
        if preconditioner is None:
            preconditioner = "illt" if self.model.local_weight < 0.999 else "identity"
        o = self._options(tolerance, max_iterations, preconditioner, precision, 0.0, triangular_sweeps)
        u = np.empty(2 * self.n_nodes)
        rep = L.SolveReport()
        L.check(self._lib.nlgpu_equilibrium_equation_2d(self._h, ctypes.byref(o), L.ptr(u), ctypes.byref(rep)))
        return u.reshape(-1, 2), SolveReport(rep.as_dict())


def equilibrium_equation(problem: MechanicalProblem2D, model: Model2D, elastic: ElasticParameters,
                         boundaries: list[MechanicalBoundary], tolerance=1e-10, **kw):
    """mechanical::equilibrium_equation (equilibrium_equation_2d.hpp:19-60): the
    displacement [n][2] of a plane-elasticity problem and the solve report."""
    problem.set_model(model)
    problem.set_elastic(elastic)
    problem.clear_mechanical_boundaries()
    for b in boundaries:
        problem.add_mechanical_boundary(b)
    if model.local_weight < 0.999:
        problem.find_neighbours()
    return problem.equilibrium(tolerance=tolerance, **kw)


def unpack_learned_weights(w) -> dict:
    """Packed parameters -> {w1 4x64, w2 128x64, w3 128x64, w4 128x1} (input x output)."""
    w = np.asarray(w, dtype=np.float64)
    o1, o2, o3 = 4 * 64, 4 * 64 + 128 * 64, 4 * 64 + 2 * 128 * 64
    return {"w1": w[:o1].reshape(4, 64), "w2": w[o1:o2].reshape(128, 64), "w3": w[o2:o3].reshape(128, 64),
            "w4": w[o3:].reshape(128, 1)}


def pack_learned_weights(d) -> np.ndarray:
    return np.concatenate([np.asarray(d[k], dtype=np.float64).ravel() for k in ("w1", "w2", "w3", "w4")]).astype(
        np.float32)


def find_neighbours(problem: Problem2D, strategy: str = "MAX"):
    """mesh::find_neighbours: widened radii, offsets, lists (reference order)."""
    r, _ = problem.find_neighbours(strategy)
    off, lst = problem.neighbours()
    return r, off, lst


def solve_assembled_batch(problems: list, tolerance: float = 1e-10, max_iterations: int = 10000,
                          check_convergence: bool = True, precision: str = "fp64"):
    """The solve stage of many assembled problems in one call
    (nlgpu_solve_assembled_batch): the non-symmetric systems (a conductivity
    field with a nonlocal model) run as one block-diagonal BiCGSTAB with
    per-instance scalars and stop tests (precision "fp64": the reference's
    diagonal preconditioner; "mixed": the FP32 ILLT of each local part), the
    others one after another.  Returns the temperatures and reports, in the
    problems' order."""
    count = len(problems)
    if count == 0:
        return [], []
    lib = problems[0]._lib
    temps = [np.empty(pb.n_nodes) for pb in problems]
    handles = (ctypes.c_void_p * count)(*[pb._h for pb in problems])
    outs = (ctypes.c_void_p * count)(*[t.ctypes.data for t in temps])
    reps = (L.SolveReport * count)()
    o = problems[0]._options(tolerance, max_iterations, "illt", precision, 0.0, 0)
    rc = lib.nlgpu_solve_assembled_batch(count, handles, ctypes.byref(o), outs, reps)
    if rc != L.OK and (check_convergence or rc != 6):
        L.check(rc)
    return temps, [SolveReport(r.as_dict()) for r in reps]


def stationary_heat_equation_solver_2d(problem: Problem2D, model: Model2D, boundaries: list[Boundary],
                                       source: float = 0.0, tolerance: float = 1e-10, max_iterations: int = 10000,
                                       preconditioner: str = "illt", precision: str = "fp64"):
    problem.set_model(model)
    problem.clear_boundaries()
    for b in boundaries:
        problem.add_boundary(b)
    if source:
        problem.set_source(source)
    return problem.stationary(tolerance, max_iterations, preconditioner, precision)


class BatchNonstationary:
    """Many nonstationary instances (each a ``NonstationaryHeatEquationSolver2D``
    after ``compute``) stepped together as one block-diagonal system."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        self._lib = L.load()
        handles = (ctypes.c_void_p * len(self.solvers))(*[s.problem.handle.value for s in self.solvers])
        self._h = ctypes.c_void_p()
        L.check(self._lib.nlgpu_batch_create(ctypes.byref(self._h), len(self.solvers), handles))

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            self._lib.nlgpu_batch_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, dirichlet_values, tolerance: float = 1e-15, max_iterations: int = 10000) -> np.ndarray:
        """One implicit-Euler step of every instance; returns each instance's CG iterations."""
        dv = L.f64(np.broadcast_to(np.asarray(dirichlet_values, dtype=np.float64), (len(self.solvers),)))
        it = np.empty(len(self.solvers), dtype=np.int64)
        L.check(self._lib.nlgpu_batch_step(self._h, L.ptr(dv), float(tolerance), int(max_iterations), L.ptr(it)))
        return it

    def temperature(self, index: int) -> np.ndarray:
        t = np.empty(self.solvers[index].problem.n_nodes)
        L.check(self._lib.nlgpu_batch_temperature(self._h, int(index), L.ptr(t)))
        return t

    def set_method(self, method: str = "identity_fp64") -> None:
        """The step's solver: "identity_fp64" (the reference's identity CG per
        instance) or "mixed_illt" (mixed-precision FCG with ILLT on the whole
        block-diagonal system, FP64 ILLT-CG fallback)."""
        L.check(self._lib.nlgpu_batch_set_method(self._h, L.BATCH_METHOD[method]))

    def last_solve(self) -> dict:
        """mixed_illt: the last step's FCG iterations, FP64 refinement steps and
        whether the FP64 ILLT-CG fallback ran."""
        inner, outer = ctypes.c_int64(), ctypes.c_int64()
        fb = ctypes.c_int()
        L.check(self._lib.nlgpu_batch_last_solve(self._h, ctypes.byref(inner), ctypes.byref(outer), ctypes.byref(fb)))
        return {"inner": inner.value, "outer": outer.value, "fallback": bool(fb.value)}

    def sizes(self) -> tuple[np.ndarray, np.ndarray]:
        """Per instance: rows and the system entries each step's SpMV reads."""
        rows = np.empty(len(self.solvers), dtype=np.int64)
        nnz = np.empty(len(self.solvers), dtype=np.int64)
        L.check(self._lib.nlgpu_batch_sizes(self._h, L.ptr(rows), L.ptr(nnz)))
        return rows, nnz


class NonstationaryHeatEquationSolver2D:
    """Implicit Euler in time: (C + dt K) T^{k+1} = C T^k + dt f, identity-preconditioned CG."""

    def __init__(self, problem: Problem2D, time_step: float):
        self.problem, self.time_step = problem, float(time_step)
        self.temperature = np.zeros(problem.n_nodes)
        self.iterations: list[int] = []

    def compute(self, initial: np.ndarray | None = None) -> None:
        init = None if initial is None else L.f64(initial)
        L.check(self.problem._lib.nlgpu_nonstationary_2d_compute(self.problem.handle, self.time_step, L.ptr(init)))
        if init is not None:
            self.temperature = init.copy()

    def calc_step(self, dirichlet_value: float = 0.0, dirichlet_values: np.ndarray | None = None,
                  tolerance: float = 1e-15, max_iterations: int = 10000) -> np.ndarray:
        dv = None if dirichlet_values is None else L.f64(dirichlet_values)
        it = ctypes.c_int64()
        t = np.empty(self.problem.n_nodes)
        rc = self.problem._lib.nlgpu_nonstationary_2d_step(self.problem.handle, float(dirichlet_value), L.ptr(dv),
                                                           float(tolerance), int(max_iterations), L.ptr(t),
                                                           ctypes.byref(it))
        if rc not in (L.OK, 6):   # the reference loops to its iteration cap without raising
            L.check(rc)
        self.iterations.append(int(it.value))
        self.temperature = t
        return t


class EigenILLTPreconditioner:
    """ILLT behind slae::preconditioner_base (preconditioner_base.hpp:8-15): the GPU
    counterpart of eigen_preconditioner with Eigen::IncompleteCholesky.

    ``compute`` factorises an upper-stored symmetric CSR (diagonal first);
    ``computation_info`` is Eigen's code (0 Success, 1 NumericalIssue);
    ``solve`` returns M^-1 x."""

    SUCCESS, NUMERICAL_ISSUE = 0, 1

    def __init__(self, context: Context | None = None):
        self.context = context if context is not None else Context()
        self._info = self.NUMERICAL_ISSUE
        self._n = 0

    def analyze_pattern(self, csr) -> "EigenILLTPreconditioner":
        return self          # the pattern is analysed by compute

    def factorize(self, csr) -> "EigenILLTPreconditioner":
        return self.compute(csr)

    def compute(self, csr) -> "EigenILLTPreconditioner":
        rp, col, val = L.i64(csr[0]), L.i64(csr[1]), L.f64(csr[2])
        n = rp.shape[0] - 1
        info = ctypes.c_int()
        L.check(self.context._lib.nlgpu_illt_compute(self.context.handle, n, L.ptr(rp), L.ptr(col), L.ptr(val),
                                                     ctypes.byref(info)))
        self._info, self._n = int(info.value), n
        return self

    def computation_info(self) -> int:
        return self._info

    def solve(self, x) -> np.ndarray:
        x = L.f64(x)
        y = np.empty_like(x)
        L.check(self.context._lib.nlgpu_illt_solve(self.context.handle, x.shape[0], L.ptr(x), L.ptr(y)))
        return y

    def solve_f32(self, x, sweeps=L.DEFAULT_TRIANGULAR_SWEEPS) -> np.ndarray:
        """M^-1 x in FP32 as the mixed-precision solve applies it: ``sweeps`` Jacobi
        sweeps per triangle, or -1 for the exact level-scheduled sweeps."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        y = np.empty_like(x)
        L.check(self.context._lib.nlgpu_illt_solve_f32(self.context.handle, x.shape[0], int(sweeps), L.ptr(x),
                                                       L.ptr(y)))
        return y


def conjugate_gradient(problem: Problem2D, a_csr, b, x0=None, preconditioner_csr=None, tolerance=1e-10,
                       max_iterations=10000):
    """slae::conjugate_gradient on an upper-stored symmetric CSR (diagonal first in each row)."""
    rp, col, val = (L.i64(a_csr[0]), L.i64(a_csr[1]), L.f64(a_csr[2]))
    b = L.f64(b)
    n = b.shape[0]
    x = np.empty(n)
    x0 = None if x0 is None else L.f64(x0)
    if preconditioner_csr is not None:
        prp, pcol, pval = (L.i64(preconditioner_csr[0]), L.i64(preconditioner_csr[1]), L.f64(preconditioner_csr[2]))
    else:
        prp = pcol = pval = None
    rep = L.SolveReport()
    rc = problem._lib.nlgpu_cg_solve(problem.handle, n, L.ptr(rp), L.ptr(col), L.ptr(val), L.ptr(prp), L.ptr(pcol),
                                     L.ptr(pval), L.ptr(b), L.ptr(x0), float(tolerance), int(max_iterations), L.ptr(x),
                                     ctypes.byref(rep))
    L.check(rc)
    return x, SolveReport(rep.as_dict())


def stationary_heat_equation_solver_1d(context: Context | None = None, elements: int = 1000, order: int = 2, length: float = 1.0,
                                       radius: float = 0.1, local_weight: float = 0.5, influence: str = "bell",
                                       conductivity: float = 1.0, t_left: float = 0.0, q_right: float = 1.0,
                                       sin_source: bool = True) -> np.ndarray:
    kinds = {"bell": 0, "triangle": 1, "normal": 2, "constant": 3}
    ctx = context if context is not None else Context()
    t = np.empty(elements * order + 1)
    L.check(ctx._lib.nlgpu_stationary_1d(ctx.handle, int(elements), int(order), float(length), float(radius),
                                             float(local_weight), kinds[influence], float(conductivity), float(t_left),
                                             float(q_right), int(bool(sin_source)), L.ptr(t)))
    return t


INFLUENCE_1D = {"bell": 0, "triangle": 1, "normal": 2, "constant": 3}


class NonstationaryHeatEquationSolver1D:
    """nonstationary_heat_equation_solver_1d<T, I> on one segment [0, length]:
    ``compute(left, right, initial)`` with each end ("temperature", value),
    ("flux", value) or ("convection", (heat_transfer, ambient_temperature))
    (the kinds are fixed by compute, as the reference's matrix portrait), then
    ``calc_step(left_value, right_value, sin_source)`` per implicit Euler step
    (a convection end's value is its ambient temperature); ``temperature`` is
    the current temperature."""

    def __init__(self, context: Context | None = None, elements: int = 200, order: int = 2, length: float = 1.0,
                 radius: float = 0.1, local_weight: float = 0.5, influence: str = "bell", conductivity: float = 1.0,
                 capacity: float = 1.0, density: float = 1.0, time_step: float = 1e-3):
        self.ctx = context if context is not None else Context()
        self.args = (int(elements), int(order), float(length), float(radius), float(local_weight),
                     INFLUENCE_1D[influence], float(conductivity), float(capacity), float(density), float(time_step))
        self.n = int(elements) * int(order) + 1
        self.time_step = float(time_step)
        self.time = 0.0

    def compute(self, left=("temperature", 0.0), right=("flux", 0.0), initial=None) -> None:
        kinds = {"temperature": L.BC_TEMPERATURE, "flux": L.BC_FLUX, "convection": L.BC_CONVECTION}
        t0 = None if initial is None else L.f64(initial)
        if t0 is not None and t0.shape != (self.n,):
            raise ValueError(f"the initial temperature needs {self.n} nodal values")
        # a convection end: (heat transfer, ambient temperature); the step value is the ambient temperature
        heat = [float(e[1][0]) if e[0] == "convection" else 0.0 for e in (left, right)]
        L.check(self.ctx._lib.nlgpu_nonstationary_1d_convection(self.ctx.handle, heat[0], heat[1]))
        nodes = ctypes.c_int64()
        L.check(self.ctx._lib.nlgpu_nonstationary_1d_compute(self.ctx.handle, *self.args, kinds[left[0]],
                                                             kinds[right[0]], L.ptr(t0), ctypes.byref(nodes)))
        assert nodes.value == self.n
        self.left, self.right = [(e[0], float(e[1][1])) if e[0] == "convection" else e for e in (left, right)]

    def calc_step(self, left_value: float | None = None, right_value: float | None = None,
                  sin_source: bool = False) -> np.ndarray:
        lv = self.left[1] if left_value is None else left_value
        rv = self.right[1] if right_value is None else right_value
        t = np.empty(self.n)
        L.check(self.ctx._lib.nlgpu_nonstationary_1d_step(self.ctx.handle, float(lv), float(rv), int(bool(sin_source)),
                                                          L.ptr(t)))
        self.time += self.time_step
        return t

    @property
    def temperature(self) -> np.ndarray:
        t = np.empty(self.n)
        L.check(self.ctx._lib.nlgpu_nonstationary_1d_temperature(self.ctx.handle, L.ptr(t)))
        return t
