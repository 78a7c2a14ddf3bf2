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
                 "b12_shuffled_cm", "s5_shuffled_cm", "b6_groups_local"]
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


def boundaries(fx: dict) -> list[tuple[int, np.ndarray, float]]:
    """(kind, edges, value) for each boundary group with a condition; kind 0 temperature, 1 flux."""
    out = []
    for key, spec in fx["config"].items():
        if not key.startswith("bc."):
            continue
        group = key[3:]
        kind, value = spec.split(":")
        val = 0.0 if value == "manufactured" else float(value)
        out.append((0 if kind == "temperature" else 1, fx["bnd_" + group], val))
    return out


def oracle_problem(fx: dict):
    """An oracle problem configured from a stationary 2D fixture (not yet solved)."""
    import oracle
    cfg = fx["config"]
    prob = oracle.Problem(element_type(fx), fx["nodes"], fx["elements"])
    prob.set_model(**model(cfg))
    for kind, edges, value in boundaries(fx):
        prob.add_boundary(kind, edges, value)
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
