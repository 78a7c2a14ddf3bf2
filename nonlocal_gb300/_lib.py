"""Loads libnlgpu.so (the sm_103a CUDA library behind include/nlgpu.h) with ctypes.

There is no CPU implementation behind this module: when the library is
missing or cannot be loaded every call raises, and compute calls need a CUDA
device.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libnlgpu.so")

c_i64, c_d, c_p, c_int = ctypes.c_int64, ctypes.c_double, ctypes.c_void_p, ctypes.c_int

OK = 0
STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "unsupported", 4: "call order violated",
          5: "numerical breakdown", 6: "no convergence", 7: "out of device memory", 8: "device wait timed out"}

BILINEAR, QUADRATIC_SERENDIPITY = 2, 3
INFLUENCE = {"constant": 0, "polynomial": 1, "exponential": 2, "fast_polynomial": 3}
CONDUCTIVITY_KIND = {1: 0, 2: 1, 3: 2}
EXPAND = {"NO": 0, "MAX": 1, "MIN": 2, "MEAN": 3}
PART_LOCAL, PART_FULL = 0, 2
BC_TEMPERATURE, BC_FLUX, BC_CONVECTION, BC_RADIATION, BC_COMBINED_FLUX = 0, 1, 2, 3, 4
ELASTIC = {"isotropic": 0, "orthotropic": 1, "anisotropic": 2}
MECH_NONE, MECH_DISPLACEMENT, MECH_PRESSURE = 0, 1, 2
MECH_CONDITION = {None: MECH_NONE, "displacement": MECH_DISPLACEMENT, "pressure": MECH_PRESSURE}
MATRIX_INNER, MATRIX_BOUND, MATRIX_LOCAL = 0, 1, 2
PRECONDITIONER = {"identity": 0, "illt": 1, "illt_learned": 2}
PRECISION = {"fp64": 0, "mixed": 1}
OPTION_GLOBAL_SWEEPS, OPTION_ORDERED_PAIRS, OPTION_ASSEMBLY_PRECISION, OPTION_FP32_SYMMETRIC = 0, 1, 2, 3
OPTION_ASSEMBLY_WARPS = 4
BATCH_METHOD = {"identity_fp64": 0, "mixed_illt": 1}
ASSEMBLY = {"auto": 0, "ff": 1, "fp64": 2}


class NlgpuError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Model2D(ctypes.Structure):
    _fields_ = [("influence", c_int), ("n", c_int), ("p", c_int), ("q", c_d), ("radius", c_d * 2),
                ("local_weight", c_d), ("conductivity_kind", c_int), ("conductivity", c_d * 3)]


class SolveOptions(ctypes.Structure):
    _fields_ = [("tolerance", c_d), ("max_iterations", c_i64), ("preconditioner", c_int), ("precision", c_int),
                ("inner_tolerance", c_d), ("triangular_sweeps", c_int), ("coarse_aggregates", c_int),
                ("coarse_aspect", c_d)]


DEFAULT_TRIANGULAR_SWEEPS = 6   # NLGPU_DEFAULT_TRIANGULAR_SWEEPS
EXACT_TRIANGULAR_SWEEPS = -1    # NLGPU_EXACT_TRIANGULAR_SWEEPS


class SolveReport(ctypes.Structure):
    _fields_ = [("iterations", c_i64), ("residual", c_d), ("reference_residual", c_d), ("preconditioner_ok", c_int),
                ("preconditioner_shifts", c_int), ("nnz_inner", c_i64), ("nnz_solver", c_i64),
                ("element_pairs", c_i64), ("seconds_neighbours", c_d), ("seconds_pattern", c_d),
                ("seconds_assembly", c_d), ("seconds_boundary", c_d), ("seconds_preconditioner", c_d),
                ("seconds_solve", c_d), ("seconds_total", c_d), ("outer_iterations", c_i64),
                ("learned_fallback", c_int), ("column_bytes", c_int), ("nonlinear_iterations", c_i64),
                ("neumann", c_int), ("nnz_fp32", c_i64), ("fp32_symmetric", c_int)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class TrainOptions(ctypes.Structure):
    _fields_ = [("right_hand_sides", c_int), ("epochs", c_int), ("batch", c_int), ("learning_rate", c_d),
                ("seed", ctypes.c_uint)]


class TrainReport(ctypes.Structure):
    _fields_ = [("samples", c_i64), ("steps", c_i64), ("loss_illt", c_d), ("loss_first", c_d), ("loss_last", c_d),
                ("seconds_harvest", c_d), ("seconds_train", c_d), ("validation_iterations_learned", c_i64),
                ("validation_iterations_illt", c_i64), ("validation_seconds_learned", c_d),
                ("validation_seconds_illt", c_d), ("learned_enabled", c_int)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


MPNN_PARAMS = 16768

# name -> (restype, argtypes); every function declared in include/nlgpu.h
SIGNATURES = {
    "nlgpu_status_string": (ctypes.c_char_p, [c_int]),
    "nlgpu_last_error": (ctypes.c_char_p, []),
    "nlgpu_device_count": (c_int, [ctypes.POINTER(c_int)]),
    "nlgpu_kernel_launches": (c_i64, []),
    "nlgpu_set_device": (c_int, [c_int]),
    "nlgpu_create": (c_int, [ctypes.POINTER(c_p), c_p]),
    "nlgpu_destroy": (c_int, [c_p]),
    "nlgpu_synchronize": (c_int, [c_p]),
    "nlgpu_mesh_2d": (c_int, [c_p, c_int, c_i64, c_p, c_i64, c_p]),
    "nlgpu_get_quadrature": (c_int, [c_p, c_p, c_p, c_p]),
    "nlgpu_get_basis": (c_int, [c_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int), c_p, c_p, c_p, c_p, c_p]),
    "nlgpu_su2_read": (c_int, [ctypes.c_char_p, ctypes.POINTER(c_p)]),
    "nlgpu_su2_free": (c_int, [c_p]),
    "nlgpu_su2_last_error": (ctypes.c_char_p, []),
    "nlgpu_su2_info": (c_int, [c_p, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), ctypes.POINTER(c_int),
                               ctypes.POINTER(c_int), ctypes.POINTER(c_int)]),
    "nlgpu_su2_nodes": (c_int, [c_p, c_p]),
    "nlgpu_su2_elements_2d": (c_int, [c_p, c_p]),
    "nlgpu_su2_group": (c_int, [c_p, c_int, c_p, c_i64, ctypes.POINTER(c_int), ctypes.POINTER(c_i64),
                                ctypes.POINTER(c_i64), ctypes.POINTER(c_int), c_p]),
    "nlgpu_cuthill_mckee": (c_int, [c_p, c_int, c_int, c_p]),
    "nlgpu_renumbering": (c_int, [c_p, c_p]),
    "nlgpu_set_model_2d": (c_int, [c_p, ctypes.POINTER(Model2D)]),
    "nlgpu_set_conductivity_field": (c_int, [c_p, c_p]),
    "nlgpu_set_capacity": (c_int, [c_p, c_d, c_d]),
    "nlgpu_find_neighbours": (c_int, [c_p, c_int, c_p, ctypes.POINTER(c_i64)]),
    "nlgpu_get_neighbours": (c_int, [c_p, c_p, c_p]),
    "nlgpu_add_boundary_2d": (c_int, [c_p, c_int, c_i64, c_int, c_p, c_d, c_p]),
    "nlgpu_add_flux_boundary_2d": (c_int, [c_p, c_int, c_i64, c_int, c_p, c_d, c_d, c_d, c_d]),
    "nlgpu_set_stationary_parameters": (c_int, [c_p, c_d, c_i64, c_d, c_p]),
    "nlgpu_get_system_rows": (c_int, [c_p, ctypes.POINTER(c_i64)]),
    "nlgpu_set_source": (c_int, [c_p, c_d, c_p]),
    "nlgpu_set_dirichlet_values": (c_int, [c_p, c_p]),
    "nlgpu_clear_boundaries": (c_int, [c_p]),
    "nlgpu_conductivity_matrix_2d": (c_int, [c_p, c_int, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)]),
    "nlgpu_get_matrix": (c_int, [c_p, c_int, c_p, c_p, c_p]),
    "nlgpu_get_rhs": (c_int, [c_p, c_p, c_p]),
    "nlgpu_stationary_2d": (c_int, [c_p, ctypes.POINTER(SolveOptions), c_p, ctypes.POINTER(SolveReport)]),
    "nlgpu_solve_assembled": (c_int, [c_p, ctypes.POINTER(SolveOptions), c_p, ctypes.POINTER(SolveReport)]),
    "nlgpu_solve_assembled_batch": (c_int, [c_i64, c_p, ctypes.POINTER(SolveOptions), c_p, c_p]),
    "nlgpu_cg_solve": (c_int, [c_p, c_i64, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_p, c_d, c_i64, c_p,
                               ctypes.POINTER(SolveReport)]),
    "nlgpu_illt_compute": (c_int, [c_p, c_i64, c_p, c_p, c_p, ctypes.POINTER(c_int)]),
    "nlgpu_illt_solve": (c_int, [c_p, c_i64, c_p, c_p]),
    "nlgpu_illt_solve_f32": (c_int, [c_p, c_i64, c_int, c_p, c_p]),
    "nlgpu_calc_flux": (c_int, [c_p, c_p, c_p, c_p]),
    "nlgpu_batch_create": (c_int, [ctypes.POINTER(c_p), c_i64, c_p]),
    "nlgpu_batch_destroy": (c_int, [c_p]),
    "nlgpu_batch_step": (c_int, [c_p, c_p, c_d, c_i64, c_p]),
    "nlgpu_batch_temperature": (c_int, [c_p, c_i64, c_p]),
    "nlgpu_batch_sizes": (c_int, [c_p, c_p, c_p]),
    "nlgpu_batch_set_method": (c_int, [c_p, c_int]),
    "nlgpu_batch_last_solve": (c_int, [c_p, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64), ctypes.POINTER(c_int)]),
    "nlgpu_nonstationary_2d_compute": (c_int, [c_p, c_d, c_p]),
    "nlgpu_nonstationary_2d_step": (c_int, [c_p, c_d, c_p, c_d, c_i64, c_p, ctypes.POINTER(c_i64)]),
    "nlgpu_stationary_1d": (c_int, [c_p, c_i64, c_int, c_d, c_d, c_d, c_int, c_d, c_d, c_d, c_int, c_p]),
    "nlgpu_nonstationary_1d_compute": (c_int, [c_p, c_i64, c_int, c_d, c_d, c_d, c_int, c_d, c_d, c_d, c_d, c_int,
                                               c_int, c_p, ctypes.POINTER(c_i64)]),
    "nlgpu_nonstationary_1d_convection": (c_int, [c_p, c_d, c_d]),
    "nlgpu_nonstationary_1d_step": (c_int, [c_p, c_d, c_d, c_int, c_p]),
    "nlgpu_nonstationary_1d_temperature": (c_int, [c_p, c_p]),
    "nlgpu_set_elastic_2d": (c_int, [c_p, c_int, c_p, c_p]),
    "nlgpu_add_mechanical_boundary_2d": (c_int, [c_p, c_i64, c_int, c_p, c_int, c_d, c_int, c_d]),
    "nlgpu_clear_mechanical_boundaries": (c_int, [c_p]),
    "nlgpu_stiffness_matrix_2d": (c_int, [c_p, c_int, ctypes.POINTER(c_i64), ctypes.POINTER(c_i64)]),
    "nlgpu_get_stiffness_matrix": (c_int, [c_p, c_int, c_p, c_p, c_p]),
    "nlgpu_get_mechanical_rhs": (c_int, [c_p, c_p, c_p]),
    "nlgpu_equilibrium_equation_2d": (c_int, [c_p, ctypes.POINTER(SolveOptions), c_p, ctypes.POINTER(SolveReport)]),
    "nlgpu_cg_solve_noalloc": (c_int, [c_p, c_i64, c_p, c_p, c_p, c_p, c_p, c_d, c_i64, ctypes.POINTER(c_i64),
                                       ctypes.POINTER(c_d)]),
    "nlgpu_set_option": (c_int, [c_p, c_int, c_int]),
    "nlgpu_assembly_tuning": (c_int, [c_p, ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_double)]),
    "nlgpu_event_record": (c_int, [c_p, c_int]),
    "nlgpu_event_elapsed": (c_int, [c_p, c_int, c_int, ctypes.POINTER(c_d)]),
    "nlgpu_flush_l2": (c_int, [c_p, c_i64]),
    "nlgpu_time_stage": (c_int, [c_p, c_int, c_int, ctypes.POINTER(c_d)]),
    "nlgpu_gemm_bf16": (c_int, [c_i64, c_int, c_i64, c_int, c_p, c_p, c_p]),
    "nlgpu_mpnn_set_weights": (c_int, [c_p, c_p]),
    "nlgpu_mpnn_set_enabled": (c_int, [c_p, c_int]),
    "nlgpu_mpnn_get_weights": (c_int, [c_p, c_p]),
    "nlgpu_mpnn_train": (c_int, [c_p, ctypes.POINTER(TrainOptions), ctypes.POINTER(TrainReport)]),
    "nlgpu_mpnn_loss_grad": (c_int, [c_p, c_p, c_p, c_p, c_p, ctypes.POINTER(c_d), c_p]),
}

_lib = None


def load(path: str = LIB_PATH) -> ctypes.CDLL:
    """Loads the library (raising if it is missing) and sets every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with nonlocal_gb300/build.py (nvcc, sm_103a)")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        msg = load().nlgpu_last_error()
        raise NlgpuError(status, msg.decode() if msg else "")


def ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def i64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int64)


def device_count() -> int:
    n = c_int(0)
    check(load().nlgpu_device_count(ctypes.byref(n)))
    return n.value


def kernel_launches() -> int:
    return int(load().nlgpu_kernel_launches())
