"""Regenerates the golden fixtures in this directory from the reference itself.

Each case writes a synthetic (or the reference's own test) mesh as SU2, runs
the reference's code on it (oracle/_ref/ref_driver, built by
oracle/build_ref.sh from the reference sources against the Eigen API shim) and
stores every dumped array plus the case configuration in ``<case>.npz``.

Runs only where the reference sources exist (the development container):

    oracle/build_ref.sh && python tests/golden/make_golden.py

The arrays are the reference's own outputs: element order is the reference
parser's (hash-set) order, so the fixtures also carry the element
connectivity the reference used.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from nonlocal_gb300.meshgen import BILINEAR, SERENDIPITY, structured_quad_mesh, write_su2  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
REFERENCE = os.environ.get("NONLOCAL_REFERENCE", "/root/reference")
REF_MESHES = os.path.join(REFERENCE, "tests", "solvers_2d", "meshes")

# name -> (mesh spec, driver arguments)
CASES = {
    # config-2 shape, scaled: bilinear, fast polynomial bell, left T=0, right flux 1
    "b12_fastpoly": ({"nx": 12, "ny": 12, "element": BILINEAR},
                     {"mode": "stationary2d", "influence": "fast_polynomial", "radius": 0.2, "local_weight": 0.5,
                      "conductivity": "1", "bc.left": "temperature:0", "bc.right": "flux:1", "tolerance": 1e-14}),
    # config-3 shape, scaled: jittered 8-node serendipity, normal kernel, orthotropic
    "s6_exp_ortho_jitter": ({"nx": 6, "ny": 6, "element": SERENDIPITY, "jitter": 0.2, "seed": 0},
                            {"mode": "stationary2d", "influence": "exponential", "n": 2, "p": 2, "q": 0.5,
                             "radius": 0.3, "local_weight": 0.3, "conductivity": "1,0.1",
                             "bc.up": "temperature:1", "bc.down": "temperature:0", "tolerance": 1e-14}),
    # general polynomial kernel, no radius widening, source term, anisotropic conductivity
    "b10_poly_no_aniso": ({"nx": 10, "ny": 8, "element": BILINEAR, "height": 0.8, "jitter": 0.15, "seed": 3},
                          {"mode": "stationary2d", "influence": "polynomial", "n": 2, "p": 4, "q": 2,
                           "radius": 0.25, "local_weight": 0.4, "conductivity": "2,1,0.5", "strategy": "NO",
                           "source": 1.5, "bc.down": "temperature:0", "bc.left": "temperature:0.5",
                           "bc.up": "flux:-1", "tolerance": 1e-14}),
    # constant kernel on serendipity, flux on two sides
    "s5_const": ({"nx": 5, "ny": 5, "element": SERENDIPITY},
                 {"mode": "stationary2d", "influence": "constant", "n": 2, "radius": 0.35, "local_weight": 0.6,
                  "conductivity": "1", "bc.left": "temperature:0", "bc.right": "flux:1", "bc.up": "flux:0.5",
                  "tolerance": 1e-14}),
    # reference's own known-answer tests (local limit)
    "ref_square16_manufactured": ({"su2": "square_1x1_16el_uniform_mesh.su2"},
                                  {"mode": "stationary2d", "local_weight": 1, "conductivity": "10,10,0",
                                   "source": "manufactured", "bc.Left": "temperature:manufactured",
                                   "bc.Right": "temperature:manufactured", "bc.Top": "temperature:manufactured",
                                   "bc.Bottom": "temperature:manufactured", "tolerance": 1e-14}),
    "ref_solid_ring": ({"su2": "solid_ring.su2"},
                       {"mode": "stationary2d", "local_weight": 1, "conductivity": "1",
                        "bc.Inner": "temperature:0", "bc.Outer": "temperature:1", "tolerance": 1e-14}),
    # spatially varying conductivity with a nonlocal model: the reference's system is
    # non-symmetric (full storage) and solved by Eigen::BiCGSTAB
    "b10_field_nonsym": ({"nx": 10, "ny": 10, "element": BILINEAR},
                         {"mode": "stationary2d", "influence": "fast_polynomial", "radius": 0.25,
                          "local_weight": 0.5, "conductivity": "1", "conductivity_field": "wave",
                          "bc.left": "temperature:0", "bc.right": "flux:1", "bc.down": "temperature:0.5"}),
    # nodes numbered at random; Cuthill-McKee of the nonlocal node graph, then the
    # whole stationary solve on the renumbered mesh (mesh_2d::renumbering)
    "b12_shuffled_cm": ({"nx": 12, "ny": 12, "element": BILINEAR, "shuffle_seed": 7},
                        {"mode": "stationary2d", "influence": "fast_polynomial", "radius": 0.2, "local_weight": 0.5,
                         "conductivity": "1", "bc.left": "temperature:0", "bc.right": "flux:1", "tolerance": 1e-14,
                         "renumber": "nonlocal"}),
    # serendipity, random numbering, renumbered by the inverse of the local-graph order
    "s5_shuffled_cm": ({"nx": 5, "ny": 5, "element": SERENDIPITY, "jitter": 0.1, "seed": 2, "shuffle_seed": 11},
                       {"mode": "stationary2d", "influence": "constant", "n": 2, "radius": 0.35, "local_weight": 0.6,
                        "conductivity": "1", "bc.left": "temperature:0", "bc.right": "flux:1", "tolerance": 1e-14,
                        "renumber": "local_reverse"}),
    # a named marker of 2D elements beside the default group (SU2 reader's group handling), local model
    "b6_groups_local": ({"nx": 6, "ny": 6, "element": BILINEAR, "groups_2d": {"inclusion": list(range(7, 21))}},
                        {"mode": "stationary2d", "local_weight": 1, "conductivity": "1", "bc.left": "temperature:0",
                         "bc.right": "flux:1", "tolerance": 1e-14}),
    # convection on the right side (convection_condition_2d + the flux alpha T_a), linear
    "b10_convection": ({"nx": 10, "ny": 10, "element": BILINEAR},
                       {"mode": "stationary2d", "influence": "fast_polynomial", "radius": 0.25, "local_weight": 0.5,
                        "conductivity": "1", "bc.left": "temperature:0", "bc.right": "convection:2,1",
                        "tolerance": 1e-14}),
    # radiation on the right side: the reference's own fixed-point loop (17 steps to 1e-8)
    "b10_radiation": ({"nx": 10, "ny": 10, "element": BILINEAR},
                      {"mode": "stationary2d", "influence": "fast_polynomial", "radius": 0.25, "local_weight": 0.5,
                       "conductivity": "20", "bc.left": "temperature:300", "bc.right": "radiation:0.5",
                       "tolerance": 1e-14}),
    # flux, convection and radiation on one side (combined_flux_2d), serendipity, constant kernel
    "s5_combined": ({"nx": 5, "ny": 5, "element": SERENDIPITY, "jitter": 0.1, "seed": 4},
                    {"mode": "stationary2d", "influence": "constant", "n": 2, "radius": 0.35, "local_weight": 0.6,
                     "conductivity": "20", "bc.left": "temperature:300", "bc.right": "combined:-100,2,280,0.3",
                     "tolerance": 1e-14}),
    # pure Neumann problems: the Lagrange row int T = energy (conductivity_matrix_2d.hpp:83-104)
    "b8_neumann": ({"nx": 8, "ny": 8, "element": BILINEAR},
                   {"mode": "stationary2d", "influence": "fast_polynomial", "radius": 0.3, "local_weight": 0.5,
                    "conductivity": "1", "bc.left": "flux:-1", "bc.right": "flux:1", "energy": 0.5,
                    "tolerance": 1e-14}),
    "s5_neumann_local": ({"nx": 5, "ny": 5, "element": SERENDIPITY, "jitter": 0.1, "seed": 4},
                         {"mode": "stationary2d", "local_weight": 1, "conductivity": "2,1", "bc.up": "flux:2",
                          "bc.down": "flux:-2", "tolerance": 1e-14}),
    # nonstationary 2D: left T = sin(10 t), identity-preconditioned CG per step
    "b8_nonstationary": ({"nx": 8, "ny": 8, "element": BILINEAR},
                         {"mode": "nonstationary2d", "influence": "fast_polynomial", "radius": 0.3,
                          "local_weight": 0.5, "conductivity": "1", "dt": 1e-3, "steps": 5, "omega": 10,
                          "dirichlet_group": "left"}),
    # nonstationary with flux, convection and radiation on the right side (radiation terms
    # of every step stay in the system matrix, as in the reference), initial T = 300
    "b8_nonstationary_radiation": ({"nx": 8, "ny": 8, "element": BILINEAR},
                                   {"mode": "nonstationary2d", "influence": "fast_polynomial", "radius": 0.3,
                                    "local_weight": 0.5, "conductivity": "1", "dt": 1e-3, "steps": 5, "omega": 10,
                                    "dirichlet_group": "left", "initial": 300,
                                    "bc.right": "combined:-1,2,0.5,0.5"}),
    # nonlocal plane elasticity (DoF = 2): left side clamped, pressure on the right side
    "m8_mechanical": ({"nx": 8, "ny": 8, "element": BILINEAR},
                      {"mode": "mechanical2d", "influence": "fast_polynomial", "radius": 0.3, "local_weight": 0.5,
                       "young_modulus": 210, "poissons_ratio": 0.3, "mbc.left": "d:0,d:0", "mbc.right": "p:1,p:0",
                       "tolerance": 1e-14}),
    "s4_mechanical_local": ({"nx": 4, "ny": 4, "element": SERENDIPITY, "jitter": 0.1, "seed": 5},
                            {"mode": "mechanical2d", "local_weight": 1, "young_modulus": 100, "poissons_ratio": 0.25,
                             "mbc.down": "d:0,d:0", "mbc.up": "p:0,p:-2", "tolerance": 1e-14}),
    # 1D stationary, the full 1000-element quadratic configuration and a small linear one
    "d1_quadratic_1000": ({"none": True},
                          {"mode": "stationary1d", "elements": 1000, "order": 2, "radius": 0.1, "local_weight": 0.5,
                           "influence": "bell", "conductivity": 1, "left_temperature": 0, "right_flux": 1,
                           "source": "sin"}),
    # 1D nonstationary (nonstationary_heat_equation_solver_1d): 5 implicit Euler steps
    "d1_nonstationary_quadratic": ({"none": True},
                                   {"mode": "nonstationary1d", "elements": 200, "order": 2, "radius": 0.1,
                                    "local_weight": 0.5, "influence": "bell", "conductivity": 1, "capacity": 1,
                                    "density": 1, "dt": 1e-2, "steps": 5, "left": "t:0", "right": "f:1",
                                    "source": "sin", "initial": "zero"}),
    "d1_nonstationary_linear": ({"none": True},
                                {"mode": "nonstationary1d", "elements": 40, "order": 1, "radius": 0.1,
                                 "local_weight": 0.3, "influence": "triangle", "conductivity": 2, "capacity": 1.5,
                                 "density": 2, "dt": 5e-3, "steps": 4, "left": "f:-0.5", "right": "t:1",
                                 "source": "none", "initial": "sin"}),
    "d1_nonstationary_convection": ({"none": True},
                                    {"mode": "nonstationary1d", "elements": 60, "order": 2, "radius": 0.15,
                                     "local_weight": 0.4, "influence": "bell", "conductivity": 1.5, "capacity": 1,
                                     "density": 1, "dt": 1e-2, "steps": 5, "left": "c:2,1", "right": "c:0.5,-0.5",
                                     "source": "sin", "initial": "sin"}),
    "d1_linear_40_triangle": ({"none": True},
                              {"mode": "stationary1d", "elements": 40, "order": 1, "quadrature": 2, "radius": 0.1,
                               "local_weight": 0.3, "influence": "triangle", "conductivity": 2,
                               "left_temperature": 1, "right_flux": 0.5, "source": "sin"}),
}


def load_dump(path: str) -> dict[str, np.ndarray]:
    out = {}
    with open(os.path.join(path, "manifest.txt")) as f:
        for line in f:
            name, dt, shape = line.split()
            arr = np.fromfile(os.path.join(path, name + ".bin"), dtype=np.dtype(dt))
            out[name] = arr.reshape([int(s) for s in shape.split(",")])
    gfile = os.path.join(path, "groups_1d.txt")
    if os.path.exists(gfile):
        with open(gfile) as f:
            out["groups_1d"] = np.array([g.strip() for g in f if g.strip()])
    return out


def run_case(name: str, mesh_spec: dict, args: dict, tmp: str) -> None:
    args = dict(args)
    if "su2" in mesh_spec:
        args["mesh"] = os.path.join(REF_MESHES, mesh_spec["su2"])
    elif "nx" in mesh_spec:
        spec = dict(mesh_spec)
        groups_2d = spec.pop("groups_2d", None)
        m = structured_quad_mesh(spec.pop("nx"), spec.pop("ny"), spec.pop("element"), **spec)
        args["mesh"] = os.path.join(tmp, name + ".su2")
        write_su2(m, args["mesh"], groups_2d)
    out = os.path.join(tmp, name)
    cmd = [DRIVER] + [f"{k}={v}" for k, v in args.items()] + [f"out={out}"]
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    data = load_dump(out)
    if "none" not in mesh_spec:
        with open(args["mesh"], "rb") as f:   # the exact file the reference parsed
            data["su2_text"] = np.frombuffer(f.read(), dtype=np.uint8)
    for k in [k for k in data if k.startswith("t_")]:
        data.pop(k)   # wall times are not golden
    cfg = {k: v for k, v in args.items() if k != "mesh"}
    cfg["mesh_spec"] = mesh_spec
    np.savez_compressed(os.path.join(HERE, name + ".npz"), config=json.dumps(cfg), **data)
    print(f"{name}: {sorted(data)}")


def main() -> None:
    if not os.path.exists(DRIVER):
        raise SystemExit("build oracle/_ref/ref_driver first (oracle/build_ref.sh)")
    only = set(sys.argv[1:])
    with tempfile.TemporaryDirectory() as tmp:
        for name, (spec, args) in CASES.items():
            if not only or name in only:
                run_case(name, spec, args, tmp)


if __name__ == "__main__":
    main()
