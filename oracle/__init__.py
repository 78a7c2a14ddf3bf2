"""ctypes wrapper of the CPU restatement (oracle/nl_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the
checker and by bench.py for its CPU baseline.  The shipped library never
imports it.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

BILINEAR, SERENDIPITY = 2, 3
INF_CONSTANT, INF_POLYNOMIAL, INF_EXPONENTIAL, INF_FAST_POLYNOMIAL = 0, 1, 2, 3
COND_ISO, COND_ORTHO, COND_ANISO = 0, 1, 2
BC_TEMPERATURE, BC_FLUX = 0, 1
STRATEGY = {"NO": 0, "MAX": 1, "MIN": 2, "MEAN": 3}

_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        c_i64, c_d, c_p, c_int = ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_int
        L.orc_create.restype = c_p
        L.orc_create.argtypes = [c_int, c_i64, c_p, c_i64, c_p]
        L.orc_destroy.argtypes = [c_p]
        L.orc_set_model.argtypes = [c_p, c_int, c_int, c_int, c_d, c_d, c_d, c_d, c_int, c_d, c_d, c_d]
        L.orc_set_conductivity_field.argtypes = [c_p, c_p]
        L.orc_set_capacity.argtypes = [c_p, c_d, c_d]
        L.orc_add_boundary.argtypes = [c_p, c_int, c_i64, c_int, c_p, c_d]
        L.orc_add_flux_boundary.argtypes = [c_p, c_int, c_i64, c_int, c_p, c_d, c_d, c_d, c_d]
        L.orc_set_stationary.argtypes = [c_p, c_d, ctypes.c_long, c_d, c_p]
        L.orc_set_source.argtypes = [c_p, c_d]
        L.orc_set_source_field.argtypes = [c_p, c_p]
        L.orc_set_dirichlet_values.argtypes = [c_p, c_p]
        L.orc_find_neighbours.argtypes = [c_p, c_int]
        L.orc_assemble_stationary.argtypes = [c_p]
        L.orc_assemble_local.argtypes = [c_p]
        L.orc_solve.argtypes = [c_p, c_int, c_d, ctypes.c_long, c_int]
        L.orc_solve.restype = c_int
        L.orc_nonstationary.argtypes = [c_p, c_d, ctypes.c_long, c_d, c_d, ctypes.c_long]
        L.orc_calc_flux.argtypes = [c_p, c_p, c_p, c_p]
        L.orc_cuthill_mckee.argtypes = [c_p, c_int, c_int, c_p]
        L.orc_cuthill_mckee.restype = c_int
        L.orc_size.argtypes = [c_p, ctypes.c_char_p]
        L.orc_size.restype = c_i64
        L.orc_get_f64.argtypes = [c_p, ctypes.c_char_p, c_p]
        L.orc_get_i64.argtypes = [c_p, ctypes.c_char_p, c_p]
        L.orc_scalar.argtypes = [c_p, ctypes.c_char_p]
        L.orc_scalar.restype = c_d
        L.orc_stationary_1d.argtypes = [c_i64, c_int, c_d, c_d, c_d, c_int, c_d, c_d, c_d, c_int, c_p]
        L.orc_stationary_1d.restype = c_int
        L.orc_threads.restype = c_int
        L.orc_set_threads.argtypes = [c_int]
        L.orc_set_record_tolerance.argtypes = [c_p, c_d]
        _lib = L
    return _lib


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


class Problem:
    """One 2D problem held by the oracle (mesh, model, boundary conditions)."""

    _F64 = {"qcoords", "jacobians", "derivatives", "centres", "rhs", "rhs_init", "solution", "history",
            "basis_qN", "basis_qNxi", "basis_qNeta", "basis_weights", "basis_centre",
            "K_inner_val", "K_bound_val", "K_local_val", "C_inner_val", "L_val", "L_scale"}

    def __init__(self, elem_type: int, nodes: np.ndarray, elements: np.ndarray):
        self._nodes = np.ascontiguousarray(nodes, dtype=np.float64)
        self._elems = np.ascontiguousarray(elements, dtype=np.int64)
        self.h = lib().orc_create(elem_type, self._nodes.shape[0], _ptr(self._nodes),
                                  self._elems.shape[0], _ptr(self._elems))
        if not self.h:
            raise ValueError("unsupported element type")
        self._keep = []

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_destroy(h)
            self.h = None

    def set_model(self, influence=INF_FAST_POLYNOMIAL, n=2, p=2, q=1.0, radius=(0.1, 0.1), local_weight=1.0,
                  cond_kind=COND_ISO, cond=(1.0, 0.0, 0.0)):
        c = list(cond) + [0.0] * (3 - len(cond))
        lib().orc_set_model(self.h, influence, n, p, q, radius[0], radius[1], local_weight, cond_kind, *c)

    def set_conductivity_field(self, values: np.ndarray):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._keep.append(v)
        lib().orc_set_conductivity_field(self.h, _ptr(v))

    def set_capacity(self, capacity=1.0, density=1.0):
        lib().orc_set_capacity(self.h, capacity, density)

    def add_boundary(self, kind: int, edges: np.ndarray, value: float):
        e = np.ascontiguousarray(edges, dtype=np.int64)
        self._keep.append(e)
        lib().orc_add_boundary(self.h, kind, e.shape[0], e.shape[1], _ptr(e), value)

    def add_flux_boundary(self, kind: int, edges: np.ndarray, flux: float = 0.0, heat_transfer: float = 0.0,
                          ambient_temperature: float = 0.0, emissivity: float = 0.0):
        """flux (1), convection (2), radiation (3) or combined (4) group."""
        e = np.ascontiguousarray(edges, dtype=np.int64)
        lib().orc_add_flux_boundary(self.h, kind, e.shape[0], e.shape[1], _ptr(e), flux, heat_transfer,
                                    ambient_temperature, emissivity)

    def set_stationary(self, tolerance: float = 1e-8, max_iterations: int = 100, energy: float = 0.0,
                       initial: np.ndarray | None = None):
        """stationary_equation_parameters_2d: the radiation loop and the Neumann energy."""
        t = None if initial is None else np.ascontiguousarray(initial, dtype=np.float64)
        if t is not None:
            self._keep.append(t)
        lib().orc_set_stationary(self.h, tolerance, max_iterations, energy, _ptr(t))

    def set_source(self, value: float):
        lib().orc_set_source(self.h, value)

    def set_source_field(self, values: np.ndarray):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._keep.append(v)
        lib().orc_set_source_field(self.h, _ptr(v))

    def set_dirichlet_values(self, values: np.ndarray):
        v = np.ascontiguousarray(values, dtype=np.float64)
        self._keep.append(v)
        lib().orc_set_dirichlet_values(self.h, _ptr(v))

    def find_neighbours(self, strategy: str = "MAX"):
        lib().orc_find_neighbours(self.h, STRATEGY[strategy])

    def assemble(self):
        lib().orc_assemble_stationary(self.h)

    def assemble_local(self):
        lib().orc_assemble_local(self.h)

    def set_record_tolerance(self, tol: float) -> None:
        """Record the CG time ("cg_to_record") and iterations ("record_iterations")
        at which later solves first reach `tol` (0: off)."""
        lib().orc_set_record_tolerance(self.h, tol)

    def solve(self, variant: int = 0, tol: float = 1e-10, maxit: int = 10000, true_residual: bool = True) -> bool:
        return bool(lib().orc_solve(self.h, variant, tol, maxit, int(true_residual)))

    def nonstationary(self, dt: float, steps: int, omega: float, tol: float = 1e-15, maxit: int = 10000):
        lib().orc_nonstationary(self.h, dt, steps, omega, tol, maxit)

    def calc_flux(self, temperature: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """heat_equation_solution_2d::calc_flux of a nodal temperature field."""
        t = np.ascontiguousarray(temperature, dtype=np.float64)
        fx, fy = np.empty_like(t), np.empty_like(t)
        lib().orc_calc_flux(self.h, _ptr(t), _ptr(fx), _ptr(fy))
        return fx, fy

    def cuthill_mckee(self, only_local: bool = False, reverse: bool = False) -> np.ndarray:
        """mesh::utils::cuthill_mckee: permutation[old] = new (inverse with reverse)."""
        out = np.empty(self._nodes.shape[0], dtype=np.int64)
        if lib().orc_cuthill_mckee(self.h, int(only_local), int(reverse), _ptr(out)) != 0:
            raise RuntimeError("node graph is not connected")
        return out

    def get(self, name: str) -> np.ndarray:
        n = lib().orc_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        if name in self._F64:
            out = np.empty(n, dtype=np.float64)
            lib().orc_get_f64(self.h, name.encode(), _ptr(out))
        else:
            out = np.empty(n, dtype=np.int64)
            lib().orc_get_i64(self.h, name.encode(), _ptr(out))
        return out

    def scalar(self, name: str) -> float:
        return lib().orc_scalar(self.h, name.encode())

    def csr(self, name: str):
        return self.get(name + "_rowptr"), self.get(name + "_col"), self.get(name + "_val")


def stationary_1d(elements=1000, order=2, length=1.0, radius=0.1, local_weight=0.5, influence="bell",
                  conductivity=1.0, t_left=0.0, q_right=1.0, sin_source=True) -> np.ndarray:
    kinds = {"bell": 0, "triangle": 1, "normal": 2, "constant": 3}
    out = np.empty(elements * order + 1, dtype=np.float64)
    rc = lib().orc_stationary_1d(elements, order, length, radius, local_weight, kinds[influence], conductivity,
                                 t_left, q_right, int(sin_source), _ptr(out))
    if rc != 0:
        raise RuntimeError("1D factorisation failed")
    return out


def threads() -> int:
    return lib().orc_threads()


def set_threads(n: int) -> None:
    lib().orc_set_threads(n)
