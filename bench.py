#!/usr/bin/env python3
"""Benchmark of the nonlocal thermal hot path on GB300.

Workload (default ``config3``): unit square, 300x300 8-node serendipity
elements with the interior corner nodes jittered by U(+-0.2h) (seed 0), 3x3
Gauss, orthotropic conductivity (1, 0.1), p1 = 0.3, normal-distribution
influence (exponential kernel, n = p = 2, q = 1/2) truncated at r = 0.05 by
the neighbour search, T = 1 on the top edge and T = 0 on the bottom edge.
``config2`` is the 200x200 bilinear problem (fast_polynomial r = 0.05,
p1 = 0.5, T = 0 left, unit flux right).  Synthetic structured meshes,
deterministic.

One step = one stationary solve from the resident mesh: neighbour search,
sparsity patterns, nonlocal + local assembly (the mixed form's nonlocal pair
blocks in float-float on the FP32 pipes, the plain form's in FP64), boundary
conditions, ILLT factorisation and the solve.  value = device time per solve
of the mixed-precision method (flexible CG in FP32 with the FP32 ILLT
application, FP64 reliable updates of the residual and solution; with the
message-passing correction when its validation gate keeps it on), by CUDA
events on the library's stream, L2 flushed between steps.  The mixed solve
stops at the workload's stop tolerance (|b - Ax| / |b| in FP64), chosen so
that its nodal error against a plain FP64 solve to 1e-13 is below 1e-9; the
error is measured and reported.  The plain FP64 ILLT-CG is timed the same
way at the metric's 1e-10 and at the mixed solve's stop tolerance.  e2e =
the same mixed solve through the C ABI from host buffers (context creation,
mesh and weights upload, temperature download included).

At N = 1 the CPU restatement of the reference (oracle/) solves the same
workload once on all host cores (the reported CPU baseline, timed to the
1e-10 residual crossing) and checks the CUDA path at full size: neighbour
lists and the inner pattern bit-exact, FP64 matrix values, and temperatures.

--impl reference times the reference algorithm on the host cores instead
(the CPU restatement in oracle/, all threads), same workload and metric.
Multi-GPU (torchrun): independent replicas, one per rank (the path does not
shard); the time is the maximum over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("time to 1e-10 relative residual, nonlocal stationary 2D solve (full pipeline): learned mixed-precision "
          "FCG vs plain FP64 ILLT-CG")
# method -> (precision, preconditioner, triangular sweeps of the FP32 ILLT: 0 the library's
# default Jacobi sweeps, -1 exact level-scheduled substitution; coarse-space correction)
METHODS = {"learned": ("mixed", "illt_learned", 0, False), "mixed": ("mixed", "illt", 0, False),
           "coarse": ("mixed", "illt", 0, True), "mixed_exact": ("mixed", "illt", -1, False),
           "plain": ("fp64", "illt", 0, False)}
METHOD_NAMES = {"learned": "mixed-precision FCG with ILLT + learned message-passing correction",
                "coarse": "mixed-precision FCG with ILLT + coarse-space (aggregation deflation) correction; the "
                          "learned message-passing correction gated off (it did not beat ILLT alone)"}


def coarse_target(n_nodes: int) -> int:
    """Aggregates of the coarse-space correction: about 160 nodes each, 64 .. 1024
    (on the 300x300 serendipity problem 1024 aggregates beat 768, 1536 and 2048:
    the FP64 Gauss-Jordan inverse grows as nc^3, the iterations fall slowly)."""
    return int(min(1024, max(64, n_nodes // 160)))
LEARNED_TRAINING = dict(right_hand_sides=2, epochs=20, batch=4, learning_rate=2e-3, seed=0)
METRIC_TOLERANCE = 1e-10      # the metric's residual
REFERENCE_TOLERANCE = 1e-13   # the FP64 solve the nodal error is measured against
NODAL_ERROR_BAR = 1e-9

WORKLOADS = {
    "config2": dict(name="200x200 bilinear, fast_polynomial r=0.05, p1=0.5, left T=0 / right flux 1",
                    nx=200, ny=200, element="bilinear", jitter=0.0,
                    model=dict(influence="fast_polynomial", radius=(0.05, 0.05), local_weight=0.5, conductivity=(1.0,)),
                    bcs=[("left", "temperature", 0.0), ("right", "flux", 1.0)], stop_tolerance=1e-10),
    "config3": dict(name="300x300 8-node serendipity jittered 0.2h, normal kernel r=0.05, p1=0.3, ortho (1,0.1), "
                         "top T=1 / bottom T=0",
                    nx=300, ny=300, element="serendipity", jitter=0.2,
                    model=dict(influence="exponential", radius=(0.05, 0.05), local_weight=0.3, conductivity=(1.0, 0.1)),
                    bcs=[("up", "temperature", 1.0), ("down", "temperature", 0.0)], stop_tolerance=1e-12),
}
DEFAULT_WORKLOAD = "config3"
# algorithmic FLOPs of one element pair: 2 D (nq^2 nen + nen nq nen), D = 2
PAIR_FLOPS = {"bilinear": 2 * 2 * (4 * 4 * 4 + 4 * 4 * 4), "serendipity": 2 * 2 * (9 * 9 * 8 + 8 * 9 * 8)}
PAIR_QUAD = {"bilinear": 16, "serendipity": 81}
L2_FLUSH_BYTES = 256 << 20
SETUP_THREADS = 16   # host threads setting up the batched workload's instances
# FP32 FMA rate of this machine's GB300 (152 SMs), measured with a CUDA-event timed
# loop of independent FMAs: 74.0 TFLOP/s (nominal 152 x 128 x 2 x 2.07 GHz = 80.5);
# the measured-peaks file holds no FP32 figure
FP32_PEAK_TFLOPS = 74.0
FP32_PEAK_KIND = "measured FP32 FMA loop (CUDA events) on GB300, 74.0 TFLOP/s; nominal 80.5"
# FP32 instructions per float-float multiply-add of the kernel's compensated
# dot products (exact product with the cross terms 4, TwoSum 6, compensation 2):
# the float-float kernel's own issue cost per algorithmic multiply-add
FF_INSTRUCTIONS = 12
# CPU arm: stop taking further full solves once this much time has gone
REFERENCE_BUDGET_S = 150.0


def peaks() -> tuple[dict, str]:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def profile_traffic() -> dict:
    """DRAM bytes per launch from the committed ncu summaries (profiles/roofline_traffic.txt)."""
    out = {}
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if os.path.exists(path):
        for line in open(path):
            parts = line.split()
            if len(parts) >= 3 and not line.startswith("#"):
                out[(parts[0], parts[1])] = float(parts[2])
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.file = None

    def start(self):
        self.file = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # let nvidia-smi finish starting up (its NVML initialisation competes with
        # the CUDA calls of the first timed steps) before the timed region begins
        deadline = time.perf_counter() + 5.0
        while time.perf_counter() < deadline and os.path.getsize(self.file.name) == 0 and self.proc.poll() is None:
            time.sleep(0.02)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.file:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        os.unlink(self.file.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, value: float) -> float:
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_problem(w, T, mesh):
    pb = T.Problem2D.from_mesh(mesh)
    pb.set_model(T.Model2D(**w["model"]))
    for group, kind, value in w["bcs"]:
        pb.add_boundary(T.Boundary(edges=mesh.boundaries[group], kind=kind, value=value))
    return pb


def cpu_solve(w, mesh, tolerance: float, record_tolerance: float = 0.0):
    """One full solve of the workload by the CPU restatement (ILLT-CG, true
    residual |b - Ax| / |b| <= tolerance).  Returns the oracle problem (kept for
    parity checks) and the timings: `seconds` the whole solve, `seconds_to_record`
    the same solve stopped at the first crossing of record_tolerance."""
    import oracle
    et = oracle.BILINEAR if w["element"] == "bilinear" else oracle.SERENDIPITY
    inf = {"fast_polynomial": oracle.INF_FAST_POLYNOMIAL, "exponential": oracle.INF_EXPONENTIAL}[w["model"]["influence"]]
    cond = tuple(w["model"]["conductivity"])
    # the same kernel parameters as the GPU model (thermal.Model2D: n = p = 2, q = 1/2
    # for the exponential kernel, 1 otherwise)
    q = 0.5 if w["model"]["influence"] == "exponential" else 1.0
    t0 = time.perf_counter()
    p = oracle.Problem(et, mesh.nodes, mesh.elements)
    p.set_model(influence=inf, n=2, p=2, q=q, radius=w["model"]["radius"], local_weight=w["model"]["local_weight"],
                cond_kind=len(cond) - 1, cond=cond + (0.0,) * (3 - len(cond)))
    for group, kind, value in w["bcs"]:
        p.add_boundary(oracle.BC_TEMPERATURE if kind == "temperature" else oracle.BC_FLUX, mesh.boundaries[group], value)
    p.set_record_tolerance(record_tolerance)
    p.find_neighbours()
    p.assemble()
    p.assemble_local()
    p.solve(variant=0, tol=tolerance, maxit=100000)
    dt = time.perf_counter() - t0
    det = {"iterations": int(p.scalar("iterations")), "neighbours_s": p.scalar("neighbours"),
           "assembly_s": p.scalar("assembly"), "assembly_local_s": p.scalar("assembly_local"), "ilt_s": p.scalar("ilt"),
           "cg_s": p.scalar("cg"), "true_residual": p.scalar("true_residual"), "threads": int(p.scalar("threads")),
           "seconds": dt}
    if record_tolerance > 0.0 and p.scalar("record_iterations") >= 0:
        det["iterations_to_record"] = int(p.scalar("record_iterations"))
        det["seconds_to_record"] = dt - det["cg_s"] + p.scalar("cg_to_record")
    return p, det


def run_reference(args, w, mesh, world, rank, dist):
    """Reference arm: the reference algorithm on the host cores (CPU restatement, all threads).
    Each step is one full solve to the metric's 1e-10 residual; steps stop once
    REFERENCE_BUDGET_S has gone (at least one), and the line says how many ran."""
    if rank != 0:
        return 0
    import oracle
    oracle.build.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    t_start = time.perf_counter()
    warm = 0
    for _ in range(args.warmup):
        if time.perf_counter() - t_start > REFERENCE_BUDGET_S / 3:
            break
        cpu_solve(w, mesh, METRIC_TOLERANCE)
        warm += 1
    times, det = [], {}
    for _ in range(args.steps):
        _, det = cpu_solve(w, mesh, METRIC_TOLERANCE)
        times.append(det["seconds"])
        if time.perf_counter() - t_start > REFERENCE_BUDGET_S:
            break
    value = sum(times) / len(times)
    line = {"metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus, "steps": len(times),
            "warmup": warm, "steps_requested": args.steps, "warmup_requested": args.warmup,
            "ms_per_step": value * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": w["name"], "mesh": f"{w['nx']}x{w['ny']} {w['element']}",
                       "tolerance": METRIC_TOLERANCE},
            "cpu_baseline": {"value": value, "unit": "s", "cores": det.get("threads", cores), "kind": "port",
                             "sample": f"one full solve of the workload per step (neighbours, assembly, local "
                                       f"assembly, ILLT, CG to {METRIC_TOLERANCE:g}) by the CPU restatement; "
                                       f"{len(times)} of {args.steps} requested steps within the "
                                       f"{REFERENCE_BUDGET_S:.0f} s budget"},
            "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "details": det}
    print(json.dumps(line))
    return 0


def rel_l2(a, b) -> float:
    import numpy as np
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def full_size_parity(pb, w, mesh, temp_primary, temp_tight) -> tuple[dict, dict]:
    """The CPU restatement solves the same workload once (to 1e-13, the time of its
    1e-10 crossing recorded) and checks the CUDA path at full size: neighbour
    lists and the inner pattern bit-exact, FP64 inner values within 1e-12 of the
    largest, the plain FP64 temperature within 1e-10 and the timed solution's
    nodal error.  Returns (cpu_baseline, parity)."""
    import numpy as np
    import oracle
    oracle.build.build()
    oracle.set_threads(os.cpu_count() or 1)
    ref, det = cpu_solve(w, mesh, REFERENCE_TOLERANCE, record_tolerance=METRIC_TOLERANCE)
    parity = {}
    off, lst = pb.neighbours()
    parity["neighbours_bit_exact"] = bool(np.array_equal(off, ref.get("neigh_offsets")) and
                                          np.array_equal(lst, ref.get("neigh_list")))
    del off, lst
    pb.set_assembly_precision("fp64")
    pb.conductivity_matrix("FULL")
    rp, col, val = pb.matrix("inner")
    pb.set_assembly_precision("auto")
    orp, ocol, oval = ref.csr("K_inner")
    parity["inner_pattern_bit_exact"] = bool(np.array_equal(rp, orp) and np.array_equal(col, ocol))
    parity["nnz_inner"] = int(rp[-1])
    if val.shape == oval.shape:
        parity["inner_values_max_rel_diff"] = float(np.abs(val - oval).max() / np.abs(oval).max())
    del rp, col, val, orp, ocol, oval
    t_ref = ref.get("solution")
    parity["oracle_true_residual"] = det["true_residual"]
    parity["plain_fp64_tight_vs_oracle_rel_l2"] = rel_l2(temp_tight, t_ref)
    parity["timed_solution_vs_oracle_rel_l2"] = rel_l2(temp_primary, t_ref)
    parity["timed_solution_nodal_error_below_1e-9"] = parity["timed_solution_vs_oracle_rel_l2"] < NODAL_ERROR_BAR
    parity["ok"] = bool(parity["neighbours_bit_exact"] and parity["inner_pattern_bit_exact"] and
                        parity.get("inner_values_max_rel_diff", 1.0) <= 1e-12 and
                        parity["plain_fp64_tight_vs_oracle_rel_l2"] <= 1e-10)
    seconds = det.get("seconds_to_record", det["seconds"])
    cpu = {"value": seconds, "unit": "s", "cores": det["threads"], "kind": "port",
           "sample": f"one full solve of the same workload (neighbours, assembly, local assembly, ILLT, CG) by the CPU "
                     f"restatement of the reference (oracle/), all host threads, timed to its first "
                     f"|b-Ax|/|b| <= {METRIC_TOLERANCE:g} (then continued to {REFERENCE_TOLERANCE:g} for the parity "
                     f"checks)",
           "iterations_to_1e-10": det.get("iterations_to_record"), "iterations_to_1e-13": det["iterations"],
           "phases_s": {k: det[k] for k in ("neighbours_s", "assembly_s", "assembly_local_s", "ilt_s")}}
    return cpu, parity


def run_gpu(args, w, mesh, world, rank, local, dist):
    import ctypes

    import numpy as np

    from nonlocal_gb300 import _lib as L
    from nonlocal_gb300 import build as nbuild
    from nonlocal_gb300 import thermal as T
    nbuild.build()
    lib = L.load()
    L.check(lib.nlgpu_set_device(local))
    pb = make_problem(w, T, mesh)
    h = pb.handle
    stop_tol = w["stop_tolerance"]

    coarse = coarse_target(pb.n_nodes)

    def step(method, tol):
        precision, pre, sweeps, with_coarse = METHODS[method]
        pb.find_neighbours()
        return pb.stationary(tolerance=tol, max_iterations=100000, precision=precision, preconditioner=pre,
                             triangular_sweeps=sweeps, check_convergence=tol >= 1e-12,
                             coarse_aggregates=coarse if with_coarse else 0)

    def timed(method, tol, count):
        """count device-timed solves (CUDA events on the library's stream), L2 flushed before each."""
        ms_steps, reports, t_ = [], [], None
        for _ in range(count):
            L.check(lib.nlgpu_flush_l2(h, L2_FLUSH_BYTES))
            L.check(lib.nlgpu_event_record(h, 0))
            t_, rep_ = step(method, tol)
            L.check(lib.nlgpu_event_record(h, 1))
            ms = ctypes.c_double()
            L.check(lib.nlgpu_event_elapsed(h, 0, 1, ctypes.byref(ms)))
            ms_steps.append(ms.value)
            reports.append(rep_)
        return max_over_ranks(dist, sum(ms_steps) / len(ms_steps)), reports[-1], t_

    few = max(1, min(args.steps, 3))
    step("plain", METRIC_TOLERANCE)
    step("mixed_exact", stop_tol)
    step("mixed", stop_tol)
    # the learned correction is trained once per operator, on pairs the plain
    # solver harvests from this system (not timed as part of a solve); its
    # validation gate decides whether the timed method uses it
    train = pb.train_learned_preconditioner(**LEARNED_TRAINING)
    learned_weights = pb.learned_weights()
    primary = "learned" if train["learned_enabled"] else "coarse"
    for _ in range(args.warmup):
        step(primary, stop_tol)
    # -------- timed region: the primary method, then the comparisons
    sampler = ClockSampler(local)
    launches0 = L.kernel_launches()
    barrier(dist)
    L.check(lib.nlgpu_synchronize(h))
    sampler.start()
    mean_ms, rep, temp = timed(primary, stop_tol, args.steps)
    L.check(lib.nlgpu_synchronize(h))
    launches = L.kernel_launches() - launches0
    plain_ms, rep_plain, temp_plain = timed("plain", METRIC_TOLERANCE, max(1, min(args.steps, 5)))
    plain_same_ms, rep_plain_same, _ = timed("plain", stop_tol, few)
    exact_ms, rep_exact, _ = timed("mixed_exact", stop_tol, few)
    mixed_ms, rep_mixed, _ = timed("mixed", stop_tol, few)
    L.check(lib.nlgpu_synchronize(h))
    clocks = sampler.stop()
    barrier(dist)
    seconds = mean_ms / 1e3
    pairs = rep.element_pairs
    iters = rep.iterations
    # the FP64 solve the nodal error is measured against (not timed)
    temp_tight, rep_tight = step("plain", REFERENCE_TOLERANCE)
    accuracy = {"reference": f"plain FP64 ILLT-CG on the GPU to |b-Ax|/|b| <= {REFERENCE_TOLERANCE:g} "
                             f"(reached {rep_tight.residual:.3g} in {rep_tight.iterations} iterations)",
                "temperature_rel_l2_vs_fp64_tight": rel_l2(temp, temp_tight),
                "plain_fp64_1e-10_temperature_rel_l2_vs_fp64_tight": rel_l2(temp_plain, temp_tight),
                "bar": NODAL_ERROR_BAR}
    accuracy["meets_bar"] = accuracy["temperature_rel_l2_vs_fp64_tight"] < NODAL_ERROR_BAR

    # -------- stage timings for the roofline (device events, this problem)
    stage_ms = {}
    for stage, name, reps in [(0, "spmv", 30), (4, "spmv32", 30), (2, "illt_apply", 5), (5, "illt_apply32", 5),
                              (6, "illt_jacobi32", 20), (1, "pair_assembly", 2), (7, "pair_assembly_ff", 2),
                              (8, "flux", 2)]:
        v = ctypes.c_double()
        L.check(lib.nlgpu_time_stage(h, stage, reps, ctypes.byref(v)))
        stage_ms[name] = v.value
    n = pb.n_nodes
    nnz_solver = rep_plain.nnz_solver
    spmv_bytes = nnz_solver * (8 + 4) + (n + 1) * 8 + 2 * n * 8
    # FP32 values and 16-bit offsets (or int32 columns), row pointers, and per row
    # x, the FP64 row sum (as FP32) and y once each; the symmetric form reads
    # the strictly upper entries only
    spmv32_bytes = rep.nnz_fp32 * (4 + rep.column_bytes) + (n + 1) * 8 + 3 * n * 4
    outer = rep.outer_iterations
    # per solve of the primary (mixed) method: inner FP32 SpMV and sweeps per inner
    # iteration (+1 start per outer step), FP64 SpMV per outer residual
    per_solve_ms = {"spmv": stage_ms["spmv"] * (outer + 1), "spmv32": stage_ms["spmv32"] * iters,
                    "illt_jacobi32": stage_ms["illt_jacobi32"] * (iters + outer),
                    "pair_assembly_ff": stage_ms["pair_assembly_ff"]}
    dominant = max(per_solve_ms, key=per_solve_ms.get)
    pk, pk_kind = peaks()
    traffic = profile_traffic()
    ff_flops = pairs * PAIR_FLOPS[w["element"]]
    ff_achieved = ff_flops / (stage_ms["pair_assembly_ff"] * 1e-3) / 1e12
    assembly_roof = {"kernel": "k_assemble_pairs_ff", "bound": "fp32", "achieved": ff_achieved,
                     "peak": FP32_PEAK_TFLOPS, "peak_kind": FP32_PEAK_KIND, "unit": "TFLOP/s",
                     "frac": ff_achieved / FP32_PEAK_TFLOPS,
                     "fp32_issue_frac": ff_achieved * FF_INSTRUCTIONS / FP32_PEAK_TFLOPS,
                     "fp32_issue_note": f"model bound: algorithmic FLOP/s x {FF_INSTRUCTIONS} FP32 instructions per "
                                        "float-float multiply-add, against the same FP32 peak",
                     "fp64_kernel_ms": stage_ms["pair_assembly"],
                     "traffic": traffic.get(("k_assemble_pairs_ff", args.workload))}
    if dominant == "pair_assembly_ff":
        roof = dict(assembly_roof)
    elif dominant in ("spmv", "spmv32"):
        nbytes = spmv_bytes if dominant == "spmv" else spmv32_bytes
        achieved = nbytes / (stage_ms[dominant] * 1e-3) / 1e9
        kname = "k_spmv" if dominant == "spmv" else ("k_spmv32_up" if rep.fp32_symmetric else "k_spmv32")
        roof = {"kernel": kname, "bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"],
                "peak_kind": pk_kind, "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                "traffic": traffic.get((kname, args.workload))}
    else:
        # k Jacobi sweeps per triangle; each reads every off-diagonal entry of its
        # triangle once (value 4 B + column 4 B) and per row the right-hand side, the
        # gathered iterate and a scale (4 + 4 + 4 B) and writes the new iterate (4 B)
        k = L.DEFAULT_TRIANGULAR_SWEEPS
        jac_bytes = k * (factor_offdiag_entries(lib, h, n) * 8 + 2 * n * 16)
        achieved = jac_bytes / (stage_ms["illt_jacobi32"] * 1e-3) / 1e9
        roof = {"kernel": "k_jacobi32", "bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"],
                "peak_kind": pk_kind, "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                "traffic": traffic.get(("k_jacobi32", args.workload)), "launches_per_application": 2 * k}
    roof["algorithmic_per_launch"] = {"spmv_bytes": spmv_bytes, "spmv32_bytes": spmv32_bytes,
                                      "pair_assembly_flops": ff_flops}
    roof["per_solve_ms"] = per_solve_ms
    roof["assembly"] = assembly_roof if dominant != "pair_assembly_ff" else None

    # -------- end to end through the C ABI from host buffers
    e2e_s = []
    h2d = mesh.nodes.nbytes + mesh.n_elements * mesh.nodes_per_element * 8 + sum(
        mesh.boundaries[g].size * 8 for g, _, _ in w["bcs"]) + (learned_weights.nbytes if primary == "learned" else 0)
    d2h = n * 8
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        pe = make_problem(w, T, mesh)
        pe.find_neighbours()
        if primary == "learned":
            pe.set_learned_weights(learned_weights, enabled=True)
        te, _ = pe.stationary(tolerance=stop_tol, max_iterations=100000, precision=METHODS[primary][0],
                              preconditioner=METHODS[primary][1],
                              coarse_aggregates=coarse if METHODS[primary][3] else 0)
        e2e_s.append(time.perf_counter() - t0)
        pe.close()
    e2e = max_over_ranks(dist, sum(e2e_s) / len(e2e_s))
    renumbering = renumbering_report(w, mesh, T, L, lib, steps=1) if rank == 0 else None

    # -------- CPU baseline and full-size parity (rank 0, N=1): the CPU restatement on the host cores
    cpu, parity = None, None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu, parity = full_size_parity(pb, w, mesh, temp, temp_tight)
        accuracy["temperature_rel_l2_vs_cpu_oracle"] = parity["timed_solution_vs_oracle_rel_l2"]
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "method": METHOD_NAMES[primary], "value": seconds, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (FP32 inner solve; float-float (FP32 pipes) nonlocal pair blocks; FP64 residual, "
                 "refinement, dots)",
        "data": "synthetic",
        "config": {"workload": w["name"], "mesh": f"{w['nx']}x{w['ny']} {w['element']}",
                   "stop_tolerance": stop_tol, "metric_tolerance": METRIC_TOLERANCE,
                   "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MiB write)",
                   "parallelism": f"replicas x{world}"},
        "accuracy": accuracy,
        "throughput": {"element_pairs_per_s": pairs / seconds,
                       "pair_quadrature_contributions_per_s": pairs * PAIR_QUAD[w["element"]] / seconds,
                       "cg_iterations_per_s": iters / seconds},
        "solve": {"element_pairs": pairs, "nnz_inner_upper": rep.nnz_inner, "nnz_solver_full_padded": nnz_solver,
                  "nnz_fp32_spmv": rep.nnz_fp32, "fp32_spmv_symmetric": rep.fp32_symmetric,
                  "cg_iterations": iters, "outer_iterations": rep.outer_iterations, "residual": rep.residual,
                  "reference_residual": rep.reference_residual,
                  "phases_s": {k: getattr(rep, "seconds_" + k) for k in
                               ["neighbours", "pattern", "assembly", "boundary", "preconditioner", "solve"]},
                  "stage_ms": stage_ms},
        "learned_training": dict(train, **{"config": LEARNED_TRAINING}),
        "coarse_aggregates": coarse if METHODS[primary][3] else 0,
        "mixed_illt": {"ms_per_step": mixed_ms, "cg_iterations": rep_mixed.iterations,
                       "reliable_updates": rep_mixed.outer_iterations, "residual": rep_mixed.residual,
                       "triangular_sweeps": L.DEFAULT_TRIANGULAR_SWEEPS,
                       "note": "the same mixed-precision FCG without the coarse-space correction (ILLT alone)"},
        "mixed_illt_exact_sweeps": {"ms_per_step": exact_ms, "cg_iterations": rep_exact.iterations,
                                    "reliable_updates": rep_exact.outer_iterations, "residual": rep_exact.residual},
        "plain_fp64": {"ms_per_step": plain_ms, "cg_iterations": rep_plain.iterations, "residual": rep_plain.residual,
                       "tolerance": METRIC_TOLERANCE},
        "plain_fp64_at_stop_tolerance": {"ms_per_step": plain_same_ms, "cg_iterations": rep_plain_same.iterations,
                                         "residual": rep_plain_same.residual, "tolerance": stop_tol},
        "speedup_vs_plain_fp64": plain_ms / mean_ms,
        "speedup_vs_plain_fp64_at_stop_tolerance": plain_same_ms / mean_ms,
        # heat_equation_solution_2d::calc_flux of the solution (FP64): local flux, the
        # nonlocal average over every ordered neighbour pair's nq x nq quadrature points
        "post_processing": {"flux_ms": stage_ms["flux"],
                            "flux_pair_quadrature_evaluations_per_s":
                                pairs * PAIR_QUAD[w["element"]] / (stage_ms["flux"] * 1e-3)},
        "renumbering": renumbering,
        "clocks": clocks,
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "cpu_baseline": cpu,
        "parity_full_size": parity,
    }
    print(json.dumps(line))
    return 0


def renumbering_report(w, mesh, T, L, lib, steps: int) -> dict:
    """The same workload with its nodes numbered at random (as an unstructured
    mesher may number them): mixed-precision solve time as numbered, the time
    of mesh::utils::cuthill_mckee (nonlocal node graph) and mesh_2d::renumbering,
    and the solve time after renumbering."""
    import ctypes
    import numpy as np
    from nonlocal_gb300.meshgen import relabel_nodes
    shuffled = relabel_nodes(mesh, np.random.default_rng(1).permutation(mesh.n_nodes))
    pb = make_problem(w, T, shuffled)
    h = pb.handle
    precision, pre, sweeps, _ = METHODS["mixed"]

    def solve_ms():
        out = []
        for k in range(steps + 1):   # the first solve after a (re)numbering is a warm-up
            pb.find_neighbours()
            L.check(lib.nlgpu_flush_l2(h, L2_FLUSH_BYTES))
            L.check(lib.nlgpu_event_record(h, 0))
            _, rep = pb.stationary(tolerance=w["stop_tolerance"], max_iterations=100000, precision=precision,
                                   preconditioner=pre, triangular_sweeps=sweeps)
            L.check(lib.nlgpu_event_record(h, 1))
            ms = ctypes.c_double()
            L.check(lib.nlgpu_event_elapsed(h, 0, 1, ctypes.byref(ms)))
            if k:
                out.append(ms.value)
        return sum(out) / len(out), rep

    before_ms, rep_before = solve_ms()
    t0 = time.perf_counter()
    perm = pb.cuthill_mckee(only_local=False, reverse=False)
    cm_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    pb.renumbering(perm)
    pb.synchronize()
    renumber_s = time.perf_counter() - t0
    after_ms, rep_after = solve_ms()
    pb.close()
    return {"numbering": "random permutation of the workload's nodes (default_rng(1))",
            "solve_ms_as_numbered": before_ms, "cg_iterations_as_numbered": rep_before.iterations,
            "cuthill_mckee_s": cm_s, "renumbering_s": renumber_s,
            "solve_ms_after_cuthill_mckee": after_ms, "cg_iterations_after": rep_after.iterations,
            "method": "mixed"}


def factor_offdiag_entries(lib, h, n: int) -> int:
    """Off-diagonal entries read by both triangular sweeps: the factor has the
    pattern of the upper local matrix, each sweep reads it once."""
    import numpy as np
    from nonlocal_gb300 import _lib as L
    rp = np.empty(n + 1, dtype=np.int64)
    L.check(lib.nlgpu_get_matrix(h, L.MATRIX_LOCAL, L.ptr(rp), None, None))
    return int(2 * (rp[-1] - n))


def batch_instances(count: int, seed: int = 0):
    """Batched nonstationary workload: meshes with edge counts ~U{64..256}, r ~ U[0.03, 0.1],
    p1 = 0.5, conductivity 1, dt = 1e-3, T = sin(10 t) on the left edge (seeded)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(64, 257)), float(rng.uniform(0.03, 0.1))) for _ in range(count)]


def config4_instances(count: int, seed: int = 0):
    """Variable-conductivity workload: 128x128 bilinear meshes, r ~ U[0.02, 0.08],
    p1 ~ U[0.2, 0.8], a log-normal conductivity exp(g) with g a Gaussian random
    field (correlation length 0.1, std 0.5), one field seed per instance."""
    import numpy as np
    rng = np.random.default_rng(seed + 4)
    return [(float(rng.uniform(0.02, 0.08)), float(rng.uniform(0.2, 0.8)), int(rng.integers(1 << 31)))
            for _ in range(count)]


def run_config4(args, world, rank, local, dist):
    """--workload config4: many variable-conductivity stationary problems.  A
    conductivity field with a nonlocal model makes the reference's system
    non-symmetric (evaluate_conductivity.hpp:9-48, stationary_heat_equation_solver_2d.hpp:105-108):
    full storage, ordered-pair assembly and Jacobi-preconditioned BiCGSTAB, as
    the reference.  A step assembles every instance (the contexts on their own
    streams from host threads) and then solves all of them as one
    block-diagonal BiCGSTAB with per-instance scalars (--solve4 batch), or
    each on its own (--solve4 single)."""
    import numpy as np
    from concurrent.futures import ThreadPoolExecutor
    from nonlocal_gb300 import _lib as L
    from nonlocal_gb300 import build as nbuild
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.fields import lognormal_conductivity
    from nonlocal_gb300.meshgen import structured_quad_mesh
    nbuild.build()
    lib = L.load()
    L.check(lib.nlgpu_set_device(local))
    tol, edges = 1e-10, 128
    specs = config4_instances(args.instances4, seed=rank)
    mesh = structured_quad_mesh(edges, edges, "bilinear")

    def make(spec):
        r, p1, seed = spec
        pb = T.Problem2D.from_mesh(mesh)
        pb.set_model(T.Model2D(influence="fast_polynomial", radius=(r, r), local_weight=p1))
        qc = pb.quadrature()[0]
        pb.set_conductivity_field(lognormal_conductivity(qc, 0.1, 0.5, seed=seed))
        pb.add_boundary(T.Boundary(edges=mesh.boundaries["left"], kind="temperature", value=0.0))
        pb.add_boundary(T.Boundary(edges=mesh.boundaries["right"], kind="flux", value=1.0))
        pb.set_assembly_precision(args.assembly4)
        pb.find_neighbours()
        return pb

    precision = "mixed" if args.precond4 == "illt" else "fp64"

    def solve(pb):
        _, rep = pb.stationary(tolerance=tol, max_iterations=100000, precision=precision)
        return rep

    def assemble(pb):
        pb.conductivity_matrix("FULL")

    solve_seconds = []

    def step(pool, prec=None):
        if args.solve4 == "single":
            return list(pool.map(solve, problems))
        list(pool.map(assemble, problems))
        t1 = time.perf_counter()
        _, reps_b = T.solve_assembled_batch(problems, tolerance=tol, max_iterations=100000, check_convergence=False,
                                            precision=prec or precision)
        solve_seconds.append(time.perf_counter() - t1)
        return reps_b

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=SETUP_THREADS) as pool:
        problems = list(pool.map(make, specs))
        setup_s = time.perf_counter() - t0
        for _ in range(args.warmup):
            step(pool)
        solve_seconds.clear()
        sampler = ClockSampler(local)
        barrier(dist)
        launches0 = L.kernel_launches()
        sampler.start()
        t_all = time.perf_counter()
        reps = []
        for _ in range(args.steps):
            reps.append(step(pool))
        total = time.perf_counter() - t_all
        clocks = sampler.stop()
        launches = L.kernel_launches() - launches0
        per = np.array(solve_seconds) if solve_seconds else None
        other = None
        if args.solve4 == "batch":   # the other preconditioner, a few steps
            other_prec = "fp64" if precision == "mixed" else "mixed"
            step(pool, other_prec)
            solve_seconds.clear()
            t2 = time.perf_counter()
            o_reps = [step(pool, other_prec) for _ in range(3)]
            o_total = time.perf_counter() - t2
            o_its = np.array([r.iterations for r in o_reps[-1]])
            other = {"preconditioner": "diagonal (the reference's)" if other_prec == "fp64" else "FP32 ILLT of the local parts",
                     "instance_solves_per_s": len(specs) * 3 / o_total, "batched_solve_s": float(np.mean(solve_seconds)),
                     "iterations": {"mean": float(o_its.mean()), "max": int(o_its.max())},
                     "converged": int(sum(r.residual <= tol for r in o_reps[-1]))}
    barrier(dist)
    total = max_over_ranks(dist, total)
    last = reps[-1]
    its = np.array([r.iterations for r in last])
    if per is None:
        per = np.array([r.seconds_total for r in last])
    solve_seconds = list(per) if args.solve4 == "batch" else []
    pairs = int(sum(r.element_pairs for r in last))
    # BiCGSTAB reads the full-row FP64 matrix twice per iteration
    spmv = sum(2 * int(r.iterations) * (int(r.nnz_solver) * 12 + (pb.n_nodes + 1) * 8 + 2 * pb.n_nodes * 8)
               for r, pb in zip(last, problems))
    pk, pk_kind = peaks()
    # over the batched solve's wall time (its vector updates and reductions
    # included), else over the whole step
    span = float(np.mean(solve_seconds)) if solve_seconds else total / args.steps
    achieved = spmv / span / 1e9
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        import oracle
        oracle.build.build()
        oracle.set_threads(os.cpu_count() or 1)
        sample = specs[:2]
        secs = 0.0
        for r, p1, seed in sample:
            pbq = make((r, p1, seed))
            qc = pbq.quadrature()[0]
            pbq.close()
            o = oracle.Problem(oracle.BILINEAR, mesh.nodes, mesh.elements)
            o.set_model(influence=oracle.INF_FAST_POLYNOMIAL, radius=(r, r), local_weight=p1)
            o.set_conductivity_field(lognormal_conductivity(qc, 0.1, 0.5, seed=seed))
            o.add_boundary(oracle.BC_TEMPERATURE, mesh.boundaries["left"], 0.0)
            o.add_flux_boundary(oracle.BC_FLUX, mesh.boundaries["right"], flux=1.0)
            t1 = time.perf_counter()
            o.find_neighbours()
            o.assemble()
            o.solve(tol=tol, maxit=100000)
            secs += time.perf_counter() - t1
        cpu = {"value": len(sample) / secs, "unit": "instance-solves/s", "cores": os.cpu_count() or 1,
               "kind": "port",
               "sample": f"{len(sample)} instances of the workload (neighbours, assembly, BiCGSTAB to {tol:g}) by the "
                         "CPU restatement of the reference on all host threads"}
    if rank != 0:
        for pb in problems:
            pb.close()
        return 0
    value = len(specs) * args.steps * world / total
    line = {
        "metric": "variable-conductivity nonlocal stationary solves: instance-solves per second (full pipeline "
                  "from the resident mesh, BiCGSTAB to |b - Ax| <= 1e-10 |b|)",
        "value": value, "unit": "instance-solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.assembly4 == "fp64" else "f64 (pair blocks in float-float on the FP32 pipes: entries within 1e-12 of FP64)",
        "data": "synthetic",
        "config": {"workload": f"{len(specs)} instances, {edges}x{edges} bilinear, log-normal conductivity exp(g), "
                               "g a Gaussian random field (correlation length 0.1, std 0.5), r ~ U[0.02, 0.08], "
                               "p1 ~ U[0.2, 0.8], fast polynomial kernel, left T = 0, unit flux right",
                   "instances": len(specs), "solve": args.solve4, "assembly": args.assembly4,
                   "preconditioner": args.precond4,
                   "parallelism": f"replicas x{world}, {SETUP_THREADS} host threads"},
        "solve_s": {"p50": float(np.percentile(per, 50)), "p99": float(np.percentile(per, 99)),
                    "what": "the batched solve of all instances per step" if args.solve4 == "batch"
                            else "one instance's assembly and solve, overlapping the others'"},
        "preconditioner": "FP32 ILLT of each instance's p1 K_local (this library's)" if precision == "mixed"
                          else "diagonal (the reference's)",
        "bicgstab_iterations": {"mean": float(its.mean()), "max": int(its.max())},
        "other_preconditioner": other,
        "residual_max": float(max(r.residual for r in last)),
        "converged": int(sum(r.residual <= tol for r in last)),
        "element_pairs_per_s": pairs * world / (total / args.steps),
        "setup_s": setup_s, "clocks": clocks, "gpu_launches": int(launches),
        "e2e": {"value": value, "unit": "instance-solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 8 * sum(pb.n_nodes for pb in problems),
                "note": "mesh and conductivity fields resident; every step copies each instance's temperature to the host"},
        "roofline": {"kernel": "k_bt_spmv (batched BiCGSTAB, full-row FP64)" if args.solve4 == "batch"
                     else "k_spmv (BiCGSTAB, full-row FP64)", "bound": "hbm", "achieved": achieved,
                     "peak": pk["hbm_gbs"], "peak_kind": pk_kind, "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
                     "traffic": None, "algorithmic_bytes_per_step": spmv,
                     "note": "SpMV bytes of the last step (matrix, row pointers, x and y per product) over "
                             + ("the batched solve's wall time" if solve_seconds else "the step's wall time")},
        "cpu_baseline": cpu,
        "learned": "not applied: the variable-conductivity operator is non-symmetric (the reference's semantics), "
                   "and the learned correction runs inside flexible CG on a symmetric operator",
    }
    print(json.dumps(line))
    for pb in problems:
        pb.close()
    return 0


def run_batch(args, world, rank, local, dist):
    """--workload config5: many nonstationary instances stepped together."""
    import numpy as np
    from nonlocal_gb300 import _lib as L
    from nonlocal_gb300 import build as nbuild
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    nbuild.build()
    lib = L.load()
    L.check(lib.nlgpu_set_device(local))
    dt, tol = 1e-3, 1e-10
    specs = batch_instances(args.instances, seed=rank)
    t0 = time.perf_counter()

    def make_instance(spec):
        edges, r = spec
        mesh = structured_quad_mesh(edges, edges, "bilinear")
        pb = T.Problem2D.from_mesh(mesh)
        pb.set_model(T.Model2D(influence="fast_polynomial", radius=(r, r), local_weight=0.5))
        pb.add_boundary(T.Boundary(edges=mesh.boundaries["left"], kind="temperature", value=0.0))
        pb.find_neighbours()
        # float-float pair blocks (within 1e-15 of the FP64 ones, max-norm) at a
        # third of the FP64 kernel's time; the steps themselves run in FP64
        pb.set_assembly_precision("ff")
        pb.set_assembly_warps(32)   # the tuner's choice on every workload; no per-instance timing
        s = T.NonstationaryHeatEquationSolver2D(pb, dt)
        s.compute()
        return s

    # every instance has its own context and stream: host threads (the library
    # releases the GIL in every call) set them up concurrently, so their GPU
    # work overlaps
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=SETUP_THREADS) as pool:
        solvers = list(pool.map(make_instance, specs))
    batch = T.BatchNonstationary(solvers)
    batch.set_method(args.batch_method)
    setup_s = time.perf_counter() - t0
    step = 0
    for _ in range(args.warmup):   # the first mixed step also factors the block-diagonal ILLT
        step += 1
        batch.step(np.full(len(specs), np.sin(10.0 * step * dt)), tolerance=tol, max_iterations=10000)
    sampler = ClockSampler(local)
    barrier(dist)
    launches0 = L.kernel_launches()
    sampler.start()
    lat, its, solves = [], [], []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        step += 1
        t1 = time.perf_counter()
        it = batch.step(np.full(len(specs), np.sin(10.0 * step * dt)), tolerance=tol, max_iterations=10000)
        lat.append(time.perf_counter() - t1)
        its.append(it)
        solves.append(batch.last_solve())
    total = time.perf_counter() - t_all
    clocks = sampler.stop()
    launches = L.kernel_launches() - launches0
    barrier(dist)
    total = max_over_ranks(dist, total)
    its = np.array(its)
    nodes = sum((e + 1) ** 2 for e, _ in specs)
    # roofline of the step: the SpMVs of the system matrix (full padded rows;
    # row pointers, x read and y written once), against the measured copy
    # bandwidth.  Identity CG: FP64 (8 + 4 bytes per entry) per instance
    # iteration.  Mixed ILLT: FP32 with 16-bit column offsets (4 + 2 bytes, FP32
    # vectors) per FCG iteration of the whole system, plus one FP64 product per
    # refinement step
    rows_i, nnz_i = batch.sizes()
    spmv64 = nnz_i * 12 + (rows_i + 1) * 8 + 2 * rows_i * 8
    spmv32 = nnz_i * 6 + (rows_i + 1) * 8 + 3 * rows_i * 4
    if args.batch_method == "mixed_illt":
        step_bytes = sum(sv["inner"] * float(spmv32.sum()) + sv["outer"] * float(spmv64.sum()) for sv in solves)
        step_bytes /= args.steps
        kname = "k_spmv32 (block-diagonal mixed FCG SpMV)"
    else:
        step_bytes = float((its * spmv64[None, :]).sum()) / args.steps
        kname = "k_bt_spmv (block-diagonal identity CG SpMV)"
    pk, pk_kind = peaks()
    achieved = step_bytes / (total / args.steps) / 1e9
    roof = {"kernel": kname, "bound": "hbm", "achieved": achieved,
            "peak": pk["hbm_gbs"], "peak_kind": pk_kind, "unit": "GB/s", "frac": achieved / pk["hbm_gbs"],
            "traffic": None, "algorithmic_bytes_per_step": step_bytes,
            "note": "SpMV bytes only, over the whole step time (right-hand sides, preconditioner and vector updates "
                    "not counted)"}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = batch_cpu_baseline(specs[:4], dt, tol)
    if rank != 0:
        return 0
    value = len(specs) * args.steps * world / total
    line = {
        "metric": "batched nonstationary 2D nonlocal steps: instance-steps per second (implicit Euler, every "
                  "instance to |b - Ax| <= 1e-10 |b|)",
        "method": ("mixed-precision FCG on the block-diagonal system, ILLT of C + dt p1 K_local (FP32 Jacobi "
                   "sweeps), FP64 reliable updates, FP64 ILLT-CG fallback" if args.batch_method == "mixed_illt"
                   else "identity-preconditioned FP64 CG per instance (the reference's per-step solve)"),
        "value": value, "unit": "instance-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64" if args.batch_method == "mixed_illt" else "f64", "data": "synthetic",
        "config": {"workload": f"{len(specs)} instances, edges ~U{{64..256}}, r ~ U[0.03, 0.1], p1 = 0.5, dt = 1e-3, "
                               "left T = sin(10 t), bilinear", "instances": len(specs), "nodes": int(nodes),
                   "parallelism": f"replicas x{world}"},
        "step_latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
        "cg_iterations": {"max_per_step": int(its.max()), "mean": float(its.mean())},
        "mixed_solves": solves if args.batch_method == "mixed_illt" else None,
        "setup_s": setup_s, "clocks": clocks, "gpu_launches": int(launches),
        "e2e": {"value": value, "unit": "instance-steps/s", "h2d_bytes_per_step": 8 * len(specs),
                "d2h_bytes_per_step": 8 * len(specs)},
        "roofline": roof, "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    batch.close()
    return 0


def batch_cpu_baseline(specs, dt: float, tol: float, steps: int = 3) -> dict:
    """The CPU restatement steps a sample of the batched workload's instances
    (the reference steps one problem at a time: identity CG per step), all host
    threads; instance-steps per second over the step loops (set-up excluded,
    as in the GPU figure)."""
    import oracle
    from nonlocal_gb300.meshgen import structured_quad_mesh
    oracle.build.build()
    oracle.set_threads(os.cpu_count() or 1)
    secs = 0.0
    for edges, r in specs:
        mesh = structured_quad_mesh(edges, edges, "bilinear")
        p = oracle.Problem(oracle.BILINEAR, mesh.nodes, mesh.elements)
        p.set_model(influence=oracle.INF_FAST_POLYNOMIAL, radius=(r, r), local_weight=0.5)
        p.add_boundary(oracle.BC_TEMPERATURE, mesh.boundaries["left"], 0.0)
        p.find_neighbours()
        p.nonstationary(dt, steps, 10.0, tol=tol, maxit=10000)
        secs += p.scalar("steps")
    return {"value": len(specs) * steps / secs, "unit": "instance-steps/s", "cores": os.cpu_count() or 1,
            "kind": "port",
            "sample": f"{len(specs)} instances of the workload ({', '.join(f'{e}x{e} r={r:.3f}' for e, r in specs)}), "
                      f"{steps} implicit Euler steps each (identity CG to {tol:g}, the reference's choice) by the CPU "
                      "restatement on all host threads; step loops timed, set-up excluded"}


ONCE_STAGES = ("assembly_fp64", "assembly_ff", "solve_mixed", "solve_coarse", "solve_fp64", "gemm_bf16")


def run_once(args) -> int:
    """One stage of one workload, once, for ncu captures of a single kernel on a
    case of the benchmark's shape: the pair assembly in FP64 or float-float, a
    whole stationary solve (mixed-precision without or with the coarse-space
    correction, or plain FP64), or the learned
    correction's tensor-core GEMM at one message-passing layer's shape (rows =
    the workload's nodes, 128 inputs, 64 outputs)."""
    from nonlocal_gb300 import build as nbuild
    from nonlocal_gb300 import thermal as T
    from nonlocal_gb300.meshgen import structured_quad_mesh
    nbuild.build()
    if args.once == "gemm_bf16":
        import numpy as np
        from nonlocal_gb300 import _lib as L
        w = WORKLOADS[args.workload]
        m = (w["nx"] + 1) * (w["ny"] + 1)
        rng = np.random.default_rng(0)
        a = (rng.standard_normal((m, 128)).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
        b = (rng.standard_normal((64, 128)).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)
        c = np.empty((m, 64), dtype=np.float32)
        L.check(L.load().nlgpu_gemm_bf16(m, 64, 128, 1, a.ctypes.data, b.ctypes.data, c.ctypes.data))
        print(json.dumps({"once": args.once, "workload": args.workload, "M": m, "N": 64, "K": 128}))
        return 0
    w = dict(WORKLOADS[args.workload])
    s = max(1, args.scale)
    w["nx"], w["ny"] = w["nx"] // s, w["ny"] // s
    w["model"] = dict(w["model"], radius=tuple(r * s for r in w["model"]["radius"]))
    mesh = structured_quad_mesh(w["nx"], w["ny"], w["element"], jitter=w["jitter"], seed=0)
    pb = make_problem(w, T, mesh)
    pb.find_neighbours()
    if args.once.startswith("assembly"):
        pb.set_assembly_precision("ff" if args.once == "assembly_ff" else "fp64")
        pb.conductivity_matrix("FULL")
        print(json.dumps({"once": args.once, "workload": args.workload, "scale": s, "element_pairs": pb.pairs}))
    else:
        mixed = args.once in ("solve_mixed", "solve_coarse")
        _, rep = pb.stationary(tolerance=w["stop_tolerance"] if mixed else METRIC_TOLERANCE, max_iterations=100000,
                               precision="mixed" if mixed else "fp64",
                               coarse_aggregates=coarse_target(pb.n_nodes) if args.once == "solve_coarse" else 0)
        print(json.dumps({"once": args.once, "workload": args.workload, "scale": s, "iterations": rep.iterations,
                          "residual": rep.residual}))
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["nlgpu", "reference"], default="nlgpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["config4", "config5"], default=DEFAULT_WORKLOAD)
    ap.add_argument("--instances4", type=int, default=64, help="config4: number of instances")
    ap.add_argument("--assembly4", choices=["ff", "fp64"], default="ff",
                    help="config4: pair blocks in float-float on the FP32 pipes, or in FP64")
    ap.add_argument("--precond4", choices=["illt", "jacobi"], default="illt",
                    help="config4: BiCGSTAB preconditioned by the FP32 ILLT of the local parts, or by the "
                         "diagonal (the reference's)")
    ap.add_argument("--solve4", choices=["batch", "single"], default="batch",
                    help="config4: one block-diagonal BiCGSTAB over all instances, or one solve per instance")
    ap.add_argument("--instances", type=int, default=256, help="config5: number of instances")
    ap.add_argument("--batch-method", choices=["mixed_illt", "identity_fp64"], default="mixed_illt",
                    help="config5: the per-step solver")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--once", choices=sorted(ONCE_STAGES),
                    help="run one stage once on the workload and exit (profiling captures)")
    ap.add_argument("--scale", type=int, default=1,
                    help="with --once: elements per edge / scale and radius x scale (same r/h, fewer pairs)")
    args = ap.parse_args()
    if args.once:
        return run_once(args)
    world, rank, local, dist = dist_setup()
    if args.workload == "config4":
        try:
            if args.impl == "reference":
                if rank == 0:
                    print(json.dumps({"impl": "reference", "unavailable": "the variable-conductivity workload has no "
                                      "CPU arm here; its line carries a CPU-port sample as cpu_baseline"}))
                return 0
            return run_config4(args, world, rank, local, dist)
        finally:
            if dist is not None:
                dist.destroy_process_group()
    if args.workload == "config5":
        try:
            if args.impl == "reference":
                if rank == 0:
                    print(json.dumps({"impl": "reference", "unavailable": "the batched workload has no CPU arm here; "
                                      "the reference steps one instance at a time"}))
                return 0
            return run_batch(args, world, rank, local, dist)
        finally:
            if dist is not None:
                dist.destroy_process_group()
    from nonlocal_gb300.meshgen import structured_quad_mesh
    w = WORKLOADS[args.workload]
    mesh = structured_quad_mesh(w["nx"], w["ny"], w["element"], jitter=w["jitter"], seed=0)
    try:
        if args.impl == "reference":
            return run_reference(args, w, mesh, world, rank, dist)
        return run_gpu(args, w, mesh, world, rank, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
