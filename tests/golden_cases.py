"""Loads the golden fixtures (tests/golden/*.npz, made from the reference by
tests/golden/make_golden.py) and turns a fixture's configuration into the
arguments of the oracle and of the CUDA path, so both run the exact inputs the
reference ran (same node numbering, same element order)."""
from __future__ import annotations

import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

STATIONARY_2D = ["b12_fastpoly", "s6_exp_ortho_jitter", "b10_poly_no_aniso", "s5_const",
                 "ref_square16_manufactured", "ref_solid_ring",
                 "b12_shuffled_cm", "s5_shuffled_cm", "b6_groups_local",
                 "b10_convection", "b10_radiation", "s5_combined", "b8_neumann", "s5_neumann_local"]
NONLOCAL_2D = ["b12_fastpoly", "s6_exp_ortho_jitter", "b10_poly_no_aniso", "s5_const"]
# every fixture made from an SU2 file (its text is stored as su2_text)
SU2_CASES = STATIONARY_2D + ["b10_field_nonsym", "b8_nonstationary"]
# mesh::utils::cuthill_mckee variants stored in the fixtures: name -> (only_local, reverse)
CUTHILL_MCKEE = {"cm_local": (True, False), "cm_local_reverse": (True, True),
                 "cm_nonlocal": (False, False), "cm_nonlocal_reverse": (False, True)}


def mesh_before_renumbering(fx: dict) -> tuple[np.ndarray, np.ndarray]:
    """Nodes and elements as the reference read them from the SU2 file: a
    fixture made with renumber=<variant> stores the renumbered mesh, whose
    permutation (cm_<variant>, permutation[old] = new) is undone here."""
    if "nodes_before_renumbering" not in fx:
        return fx["nodes"], fx["elements"]
    p = fx["cm_" + fx["config"]["renumber"]]
    inverse = np.empty_like(p)
    inverse[p] = np.arange(p.size)
    return fx["nodes_before_renumbering"], inverse[fx["elements"]]


def lagrange_column(fx: dict) -> np.ndarray:
    """int N_i over the elements of each node (conductivity_matrix_2d.hpp:75-104), from
    the fixture's basis tables and Jacobians."""
    nen = fx["elements"].shape[1]
    qN = fx["basis_qN"].reshape(nen, -1)
    per = (fx["basis_weights"][None, None, :] * qN[None, :, :] * fx["jacobians"][:, None, :]).sum(axis=2)
    b = np.zeros(fx["nodes"].shape[0])
    np.add.at(b, fx["elements"], per)
    return b


def bordered(rp, col, val, b):
    """A pure Neumann problem's matrix as the reference stores it: every row ends with
    the Lagrange column n (b_i), row n holds a zero diagonal."""
    n = rp.shape[0] - 1
    rows_c = [np.append(col[rp[r]:rp[r + 1]], n) for r in range(n)] + [np.array([n])]
    rows_v = [np.append(val[rp[r]:rp[r + 1]], b[r]) for r in range(n)] + [np.array([0.0])]
    new_rp = np.concatenate([[0], np.cumsum([len(c) for c in rows_c])]).astype(np.int64)
    return new_rp, np.concatenate(rows_c).astype(np.int64), np.concatenate(rows_v)


def neumann(fx: dict) -> bool:
    """The fixture is a pure Neumann problem (its matrices carry the Lagrange row)."""
    return fx["K_inner_rowptr"].shape[0] == fx["nodes"].shape[0] + 2


def write_su2_text(fx: dict, path: str) -> str:
    """Writes the exact SU2 file the reference parsed for this fixture."""
    with open(path, "wb") as f:
        f.write(fx["su2_text"].tobytes())
    return path

INFLUENCE = {"constant": 0, "polynomial": 1, "exponential": 2, "fast_polynomial": 3}


def load(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        data = {k: z[k] for k in z.files}
    data["config"] = json.loads(str(data["config"]))
    if "temperature" in data and "nodes" in data and data["temperature"].shape[0] == data["nodes"].shape[0] + 1:
        # a pure Neumann problem's solution ends with the Lagrange multiplier
        data["lagrange_multiplier"] = data["temperature"][-1:]
        data["temperature"] = data["temperature"][:-1]
    return data


def element_type(fx: dict) -> int:
    return 2 if fx["elements"].shape[1] == 4 else 3


def conductivity(cfg: dict) -> tuple[int, tuple[float, float, float]]:
    vals = [float(v) for v in str(cfg.get("conductivity", "1")).split(",")]
    kind = {1: 0, 2: 1, 3: 2}[len(vals)]
    return kind, tuple(vals + [0.0] * (3 - len(vals)))


def model(cfg: dict) -> dict:
    """Influence/model arguments shared by the oracle and the CUDA path."""
    r = float(cfg.get("radius", 0.1))
    kind, cond = conductivity(cfg)
    return dict(influence=INFLUENCE[cfg.get("influence", "fast_polynomial")], n=int(cfg.get("n", 2)),
                p=int(cfg.get("p", 2)), q=float(cfg.get("q", 1.0 if cfg.get("influence") != "exponential" else 0.5)),
                radius=(r, float(cfg.get("radius2", r))), local_weight=float(cfg.get("local_weight", 1.0)),
                cond_kind=kind, cond=cond)


BOUNDARY_KINDS = {"temperature": 0, "flux": 1, "convection": 2, "radiation": 3, "combined": 4}


def boundary_specs(fx: dict) -> list[dict]:
    """Each boundary group with a condition, as the fixture's configuration gives it
    (temperature:v | flux:q | convection:alpha,T_a | radiation:eps | combined:q,alpha,T_a,eps)."""
    out = []
    for key, spec in fx["config"].items():
        if not key.startswith("bc."):
            continue
        group = key[3:]
        kind, args = spec.split(":")
        a = [0.0] if args == "manufactured" else [float(v) for v in args.split(",")]
        d = {"kind": kind, "edges": fx["bnd_" + group], "value": 0.0, "heat_transfer": 0.0,
             "ambient_temperature": 0.0, "emissivity": 0.0}
        if kind in ("temperature", "flux"):
            d["value"] = a[0]
        elif kind == "convection":
            d["heat_transfer"], d["ambient_temperature"] = a
        elif kind == "radiation":
            d["emissivity"] = a[0]
        else:
            d["value"], d["heat_transfer"], d["ambient_temperature"], d["emissivity"] = a
        out.append(d)
    return out


def boundaries(fx: dict) -> list[tuple[int, np.ndarray, float]]:
    """(kind, edges, value) for each temperature (0) or flux (1) group."""
    return [(BOUNDARY_KINDS[d["kind"]], d["edges"], d["value"]) for d in boundary_specs(fx)]


def stationary_parameters(cfg: dict) -> dict:
    """stationary_equation_parameters_2d of a fixture (defaults 1e-8, 100, 0)."""
    return {"tolerance": float(cfg.get("nonlinear_tolerance", 1e-8)),
            "max_iterations": int(cfg.get("nonlinear_max_iterations", 100)), "energy": float(cfg.get("energy", 0.0))}


def oracle_problem(fx: dict):
    """An oracle problem configured from a stationary 2D fixture (not yet solved)."""
    import oracle
    cfg = fx["config"]
    prob = oracle.Problem(element_type(fx), fx["nodes"], fx["elements"])
    prob.set_model(**model(cfg))
    for d in boundary_specs(fx):
        if d["kind"] == "temperature":
            prob.add_boundary(0, d["edges"], d["value"])
        else:
            prob.add_flux_boundary(BOUNDARY_KINDS[d["kind"]], d["edges"], d["value"], d["heat_transfer"],
                                   d["ambient_temperature"], d["emissivity"])
    p = stationary_parameters(cfg)
    prob.set_stationary(p["tolerance"], p["max_iterations"], p["energy"])
    if cfg.get("source") == "manufactured":
        prob.set_source_field(fx["source_q"].reshape(-1))
    elif "source" in cfg:
        prob.set_source(float(cfg["source"]))
    if "dirichlet_values" in fx:
        prob.set_dirichlet_values(fx["dirichlet_values"])
    return prob


def csr_to_dense(rowptr, col, val, n_rows, n_cols):
    a = np.zeros((n_rows, n_cols))
    for r in range(n_rows):
        for k in range(int(rowptr[r]), int(rowptr[r + 1])):
            a[r, int(col[k])] += val[k]
    return a
