#!/usr/bin/env python
"""p' solves/s on the 128^3 jittered-hex pressure-correction system.

Workload: the seeded 128^3 hex p' system (n = 2,097,152, 7-point, 14,581,760
real nonzeros plus the reference's phantom column on 96,776 boundary rows),
Peclet <= 10, diagonal dominance U[1.01, 1.1], RHS U[-1, 1], x0 = 0.  A step
is one complete solve to ||b - A x|| / ||b|| <= 1e-10, ILU factorisation
included (the reference refactors on every solve() call because the values
change every SIMPLE iteration).

Headline (`value`): the FP32-inner / FP64-refined ILU-BiCGSTAB, inputs resident
in HBM.  Also reported: the plain FP64 ILU-BiCGSTAB on the same system, the
reference-faithful solve() (3 fixed iterations), SpMV GB/s in both precisions,
the end-to-end rate through ocsl_solve with pinned host buffers (`e2e`) and
with pageable ones (`e2e_pageable`, what the C++ drop-in's std::vectors are), the
roofline of the dominant kernel from CUDA events recorded around every launch
during the timed region, and the reference algorithm's CPU rate on the host
cores (the oracle's OpenMP port of ILU_BICGSTAB_solve; the reference itself
cannot reach 1e-10, so a reference "solve" is its own fixed 3-iteration call).
`multicolour_ordering`: the same solves through ocsl_set_ordering's
multicolour ordering (red-black on this machine; one sweep level per colour, a
different ILU(0) factor than the reference's, so never the headline), and
natural against multicolour on the tet 64^3 x 6 p' system.

Also on rank 0 (`simple_iteration`): the reference's own CPU-runnable case end
to end -- the 1000-cell shock tube's 200 steps x 5 SIMPLE inner iterations as
device iterations (one CUDA graph each), their time per inner iteration, the
final fields against the reference's recorded ones, and the oracle's C
restatement of the same iteration timed on one host core.

`--impl reference` times only that CPU implementation (rank 0).  Multi-GPU:
independent replicas, one per rank, no collective on the data path.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "p' solves/s & SpMV HBM GB/s: FP32-IR vs plain FP64 GPU at 1e-10 rel. residual"
UNIT = "solves/s"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--flow-size", type=int, default=128,
                    help="N of the N^3 SIMPLE-iteration case (0: skip it)")
    ap.add_argument("--flow-inner", type=int, default=5)
    ap.add_argument("--tet-size", type=int, default=64,
                    help="N of the N^3 x 6 tet system of the ordering comparison (0: skip it)")
    return ap.parse_args()


def workload_config(size, n, nnz, nnz_real):
    return {"workload": f"hex{size}^3 jittered p' system, ILU-BiCGSTAB to 1e-10, x0=0",
            "n": n, "nnz_stored": nnz, "nnz_real": nnz_real, "peclet_max": 10,
            "diag_ratio": "U[1.01,1.1]", "seed": 20261203,
            "l2": f"no flush: solve working set > {L2_BYTES >> 20} MB L2",
            "parallelism": "replicas"}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic():
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    return json.load(open(p)) if os.path.isfile(p) else {}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        for line in open(self.file.name):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def lu_counts(rp, col):
    n = rp.size - 1
    rows = np.repeat(np.arange(n, dtype=np.int64), np.diff(rp.astype(np.int64)))
    c = col.astype(np.int64)  # phantom -> -1
    real = c >= 0
    lower = int(np.count_nonzero(real & (c < rows)))
    upper = int(np.count_nonzero(real & (c > rows)))
    return lower, upper


def algorithmic_bytes(n, nnz_real, nnz_l, nnz_u, structured):
    """Bytes each kernel must move per launch, by category.

    SpMV (int32 CSR): values and columns once, row pointers, x once, y, and
    the one vector its fused dot reads; on a box pattern (stencil records) no
    index at all: values, x, y and the dot's vector.  Level-scheduled sweeps
    (CSR): strict lower / upper values and columns, row pointers, diagonal
    positions (and the reciprocal diagonal backward), rhs, result.
    Structured sweeps read no indices: the strict lower / upper values, rhs,
    result (and the reciprocal diagonal backward).
    """
    out = {
        "spmv_f32": 8 * nnz_real + 4 * (n + 1) + 12 * n,
        "spmv_f64": 12 * nnz_real + 4 * (n + 1) + 24 * n,
    }
    if structured:
        out.update({"spmv_f32": 4 * nnz_real + 12 * n, "spmv_f64": 8 * nnz_real + 24 * n})
        out.update({"fw_sweep_f32": 4 * nnz_l + 8 * n, "bw_sweep_f32": 4 * nnz_u + 12 * n,
                    "fw_sweep_f64": 8 * nnz_l + 16 * n, "bw_sweep_f64": 8 * nnz_u + 24 * n})
    else:
        out.update({"fw_sweep_f32": 8 * nnz_l + 4 * (n + 1) + 12 * n,
                    "fw_sweep_f64": 12 * nnz_l + 4 * (n + 1) + 20 * n,
                    "bw_sweep_f32": 8 * nnz_u + 4 * (n + 1) + 16 * n,
                    "bw_sweep_f64": 12 * nnz_u + 4 * (n + 1) + 28 * n})
    return out


def cpu_reference_rate(sysm, seconds, threads, max_calls=None):
    """The oracle's OpenMP port of ILU_BICGSTAB_solve (cmatrix_solver.cpp:682)."""
    from oracle.oracle import Oracle

    o = Oracle()
    o.set_threads(threads)
    x0 = np.zeros(sysm.n)
    calls, t0 = 0, time.perf_counter()
    while True:
        o.bicgstab_ref(sysm.row_ptr, sysm.column_index, sysm.value, sysm.b, x0)
        calls += 1
        el = time.perf_counter() - t0
        if el >= seconds or (max_calls and calls >= max_calls):
            break
    return calls / el, calls, el


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from opencslsolver_gb300 import workloads as W
    from oracle import oracle as orc

    if not os.path.isfile(orc.ORACLE_SO):
        orc.build()
    threads = os.cpu_count() or 1
    s = W.hex_pprime(args.size, peclet=10.0)
    from oracle.oracle import Oracle

    o = Oracle()
    o.set_threads(threads)
    x0 = np.zeros(s.n)
    for _ in range(args.warmup):
        o.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        o.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
        times.append(time.perf_counter() - t0)
    ms = 1000 * sum(times) / len(times)
    v = 1000.0 / ms
    kind = "port"
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": workload_config(args.size, s.n, s.nnz, s.nnz_real),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": "one step = one full reference ILU_BICGSTAB_solve() call "
                                   "(ILU + 3 fixed iterations, the reference's own solve; it "
                                   f"cannot reach 1e-10) on the {args.size}^3 system, OpenMP "
                                   "port of cmatrix_solver.cpp:682-762"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def simple_iteration(torch, dev, cpu_inner=50):
    """The reference's own CPU-runnable case end to end: the 1000-cell shock
    tube (200 steps x 5 inner iterations, momentum through CG_solve, p' and
    enthalpy through ILU_BICGSTAB_solve) as ocsl_flow_iterate_device calls,
    one CUDA graph per inner iteration, from the reference's recorded initial
    state; the final fields against the reference's recorded ones; and the
    oracle's C restatement of the same iteration on one host core for a
    bounded number of inner iterations."""
    import opencslsolver_gb300 as ocsl
    from oracle import oracle as orc

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import flow_cases as FC

    g = FC.Golden("shocktube")
    methods = (ocsl.CG_REF, ocsl.BICGSTAB_REF, ocsl.BICGSTAB_REF)
    ctx = ocsl.Context(dev.index)
    try:
        case = FC.DeviceCase(torch, g.case())
        case.bind(ctx)
        stream = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e0.record(stream)
        for _ in range(g.steps):
            for _ in range(g.inner):
                rep = case.iterate(ctx, methods)
                assert rep["status"] == [0] * 5, rep
            case.end_step(ctx)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        iters = g.steps * g.inner
        errs = FC.field_errors(case.written(), FC.recorded(g.setup, g.record("final_cg")))
    finally:
        ctx.close()
    # the oracle's restatement on one host core, a bounded sample from the start
    cpu_case = g.case()
    orc.Oracle().set_threads(1)
    t0 = time.perf_counter()
    for k in range(cpu_inner):
        orc.flow_iterate(cpu_case, methods)
        if k % g.inner == g.inner - 1:
            FC.end_step(cpu_case, orc.flow_end_step)
    cpu_ms = 1000.0 * (time.perf_counter() - t0) / cpu_inner
    return {
        "workload": "1D shock tube, 1000 cells, 200 steps x 5 inner iterations, momentum "
                    "CG_solve, p' and enthalpy ILU_BICGSTAB_solve (reference-faithful)",
        "gpu_ms_per_inner_iteration": 1000.0 * wall / iters,
        "gpu_event_ms_per_inner_iteration": e0.elapsed_time(e1) / iters,
        "cpu_port_ms_per_inner_iteration": cpu_ms,
        "cpu_port": f"oracle C restatement of the same iteration, 1 core, first {cpu_inner} "
                    "inner iterations",
        "max_rel_err_vs_reference": {"state": max(errs[k] for k in
                                                  ("velocity", "pressure", "temperature",
                                                   "density_c", "enthalpy")),
                                     "all_fields": max(errs.values())},
        "graph": "one CUDA graph per inner iteration (captured on the second call)",
    }


def simple_iteration_at_scale(size, inner, cpu_inner=1):
    """The same iteration at scale: an N^3 hex box from an SU2 file through the
    library's reader, pattern builder and initial state (flow_bench), device
    iterations with each solver choice, and the oracle's C restatement with the
    reference's solvers on every host core for ``cpu_inner`` iterations."""
    from opencslsolver_gb300 import flow as F
    from opencslsolver_gb300 import flow_bench as FB
    from oracle import oracle as orc

    case, info = FB.box_case(size)
    info["gpu"] = FB.time_gpu(case, inner)
    cores = os.cpu_count() or 1
    orc.Oracle().set_threads(cores)
    cpu_case = F.initial_state({k: v for k, v in _mesh_of(case).items()}, **FB.CONFIG)
    t0 = time.perf_counter()
    for _ in range(cpu_inner):
        orc.flow_iterate(cpu_case, FB.methods()["reference_solvers"])
    cpu_ms = 1000.0 * (time.perf_counter() - t0) / cpu_inner
    info["cpu_port"] = {"ms_per_inner_iteration": round(cpu_ms, 1), "cores": cores,
                        "sample": f"{cpu_inner} inner iteration(s) of the oracle's C "
                                  "restatement, reference's solvers (face loops on one thread, "
                                  "solves on every core)"}
    info["speedup_reference_solvers"] = round(
        cpu_ms / info["gpu"]["reference_solvers"]["ms_per_inner_iteration"], 1)
    return info


def _mesh_of(case):
    """The mesh arrays an initial_state case was built from."""
    st, ar = case["state"], case["arrays"]
    return {"n_cells": st["volume"].size, "n_faces": case["left"].size,
            "n_bc": case["bc_left"].size, "face_left": case["left"], "face_right": case["right"],
            "bc_left": case["bc_left"], "bc_marker": case["bc_marker"],
            "face_geo_aver": st["geo_aver"], "face_ksi_A": st["ksi_A"],
            "face_area_vector": ar["face_area_vector"], "face_alpha": ar["face_alpha"],
            "face_distance": ar["face_distance"], "face_unit": ar["face_unit"],
            "bc_area": st["bc_area"], "bc_area_vector": st["bc_area_vector"],
            "bc_alpha": ar["bc_alpha"], "bc_distance": ar["bc_distance"], "bc_unit": ar["bc_unit"],
            "bc_perp_dist": st["bc_perp_dist"], "bc_ksi_A": st["bc_ksi_A"],
            "cell_volume": st["volume"], "row_ptr": case["row_ptr"],
            "column_index": case["column_index"]}


def ordering_comparison(torch, dev, stream, size, warmup, steps, tol):
    """Natural against multicolour ordering on the size^3 x 6 tet p' system
    (Peclet <= 50): ms per solve (CUDA events) for the FP32-inner and the
    FP64 ILU-BiCGSTAB to tol, iterations and true relative residuals."""
    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import workloads as W

    t = W.tet_pprime(size, peclet=50.0)
    ctx = ocsl.Context(dev.index)
    ctx.set_pattern(t.row_ptr, t.column_index)
    ctx.set_stream(stream.cuda_stream)
    A = torch.from_numpy(t.value).to(dev)
    B = torch.from_numpy(t.b).to(dev)
    X = torch.zeros(t.n, dtype=torch.float64, device=dev)
    out = {"workload": f"tet {size}^3 x 6 jittered p' system ({t.n} cells), ILU-BiCGSTAB to "
                       f"{tol:g}, x0=0"}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    try:
        for ordering in ("natural", "multicolour"):
            ctx.set_ordering(ordering)
            for name, method in (("ir32", ocsl.ILU_BICGSTAB_IR32), ("fp64", ocsl.ILU_BICGSTAB)):
                for k in range(warmup + steps):
                    if k == warmup:
                        torch.cuda.synchronize(dev)
                        e0.record(stream)
                    X.zero_()
                    r = ctx.solve_device(method, A, B, X, tol=tol)
                    if r["status"] != 0:
                        raise RuntimeError(f"tet solve failed: {r}")
                e1.record(stream)
                torch.cuda.synchronize(dev)
                out[f"{ordering}_{name}"] = {"ms_per_solve": round(e0.elapsed_time(e1) / steps, 3),
                                             "iterations": r["iterations"],
                                             "relres": r["residual"]}
        out["colours"] = ctx.ordering_info()["colours"]
        out["natural_sweep_levels"] = ctx.pattern_info()["fw_levels"]
        out["speedup_ir32"] = round(out["natural_ir32"]["ms_per_solve"] /
                                    out["multicolour_ir32"]["ms_per_solve"], 2)
    finally:
        ctx.close()
    return out


def run_ours(args):
    import torch

    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import workloads as W

    from opencslsolver_gb300.replicas import ReplicaGroup

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    group = ReplicaGroup("nccl", device=dev)
    world, rank = group.world, group.rank

    t_gen = time.perf_counter()
    s = W.hex_pprime(args.size, peclet=10.0)
    t_gen = time.perf_counter() - t_gen
    nnz_l, nnz_u = lu_counts(s.row_ptr, s.column_index.astype(np.int64))

    ctx = ocsl.Context(local)
    t_pat = time.perf_counter()
    ctx.set_pattern(s.row_ptr, s.column_index)
    t_pat = time.perf_counter() - t_pat
    # a created stream (not the legacy default one), so the library can replay
    # its iteration batches from CUDA graphs; torch works on the same stream
    torch.cuda.set_stream(torch.cuda.Stream(device=dev))
    stream = torch.cuda.current_stream(dev)
    ctx.set_stream(stream.cuda_stream)
    A = torch.from_numpy(s.value).to(dev)
    B = torch.from_numpy(s.b).to(dev)
    X = torch.zeros(s.n, dtype=torch.float64, device=dev)
    # sweep tile for this matrix (setup, before any timed region)
    t_tune = time.perf_counter()
    tune = ctx.autotune(ocsl.ILU_BICGSTAB_IR32, A)   # FP32 sweeps (headline)
    tune64 = ctx.autotune(ocsl.ILU_BICGSTAB, A)       # FP64 sweeps (plain FP64 solve)
    t_tune = time.perf_counter() - t_tune

    def solve(method):
        X.zero_()
        r = ctx.solve_device(method, A, B, X, tol=args.tol)
        if r["status"] != 0:
            raise RuntimeError(f"solve failed: {r}")
        return r

    barrier = group.barrier
    max_over_ranks = group.max_over_ranks

    def timed(method, steps, profile=False):
        for _ in range(args.warmup):
            solve(method)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        its = []
        barrier()
        torch.cuda.synchronize(dev)
        if profile:
            ctx.profile(True)
            ctx.profile_read()
        e0.record(stream)
        for _ in range(steps):
            r = solve(method)
            its.append((r["iterations"], r["outer_iterations"], r["residual"]))
        e1.record(stream)
        torch.cuda.synchronize(dev)
        barrier()
        prof = None
        if profile:
            prof = ctx.profile_read()
            ctx.profile(False)
        ms = e0.elapsed_time(e1) / steps
        return max_over_ranks(ms), its, prof

    # ---- headline: FP32-inner / FP64-refined (no per-launch events: iteration
    # batches replay from CUDA graphs as in production use)
    clocks = Clocks(local)
    clocks.start()
    ms_ir, its_ir, _ = timed(ocsl.ILU_BICGSTAB_IR32, args.steps)
    clk = clocks.stop()
    value = group.job_rate(ms_ir)
    # the same solves again with every launch bracketed by CUDA events on the
    # library's stream: per-kernel times for the roofline
    ms_ir_prof, _, prof_ir = timed(ocsl.ILU_BICGSTAB_IR32, args.steps, profile=True)

    # ---- plain FP64 GPU solve, same system and tolerance
    ms_64, its_64, _ = timed(ocsl.ILU_BICGSTAB, max(3, args.steps // 2))
    _, _, prof_64 = timed(ocsl.ILU_BICGSTAB, max(3, args.steps // 2), profile=True)
    # ---- reference-faithful solve() (ILU + 3 fixed iterations)
    ms_ref, _, _ = timed(ocsl.BICGSTAB_REF, max(3, args.steps // 2))
    # ---- the multicolour ordering: an option beside the headline (its ILU(0)
    # factor is that of the permuted system, not the reference's natural one)
    ctx.set_ordering("multicolour")
    ms_mc_ir, its_mc_ir, _ = timed(ocsl.ILU_BICGSTAB_IR32, args.steps)
    _, _, prof_mc = timed(ocsl.ILU_BICGSTAB_IR32, max(3, args.steps // 2), profile=True)
    ms_mc_64, its_mc_64, _ = timed(ocsl.ILU_BICGSTAB, max(3, args.steps // 2))
    mc_info = ctx.ordering_info()
    ctx.set_ordering("natural")
    multicolour = {"ir32_solves_per_s": world * 1000.0 / ms_mc_ir,
                   "fp64_solves_per_s": world * 1000.0 / ms_mc_64,
                   "iterations": {"ir32_inner": its_mc_ir[-1][0], "ir32_outer": its_mc_ir[-1][1],
                                  "fp64": its_mc_64[-1][0]},
                   "relres": {"ir32": its_mc_ir[-1][2], "fp64": its_mc_64[-1][2]},
                   "colours": mc_info["colours"], "sweep_levels": mc_info["levels"],
                   "stencil_records": mc_info["stencil"],
                   # per-launch CUDA-event times of the FP32-refined solves
                   # (the red-black preconditioner is accounted to fw_sweep)
                   "kernel_us_per_launch": {k: round(1000.0 * v[0] / v[1], 2)
                                            for k, v in prof_mc.items() if v[1]}}
    if args.tet_size > 0 and rank == 0:
        multicolour["tet"] = ordering_comparison(torch, dev, stream, args.tet_size, args.warmup,
                                                 max(3, args.steps // 2), args.tol)

    # ---- e2e: ocsl_solve with pinned host buffers (H2D of A, b, x0; D2H of x)
    hA = torch.from_numpy(s.value).pin_memory().numpy()
    hB = torch.from_numpy(s.b).pin_memory().numpy()
    hX = torch.zeros(s.n, dtype=torch.float64).pin_memory().numpy()
    for _ in range(args.warmup):
        hX[:] = 0.0
        ctx.solve(ocsl.ILU_BICGSTAB_IR32, hA, hB, hX, tol=args.tol)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        hX[:] = 0.0
        r = ctx.solve(ocsl.ILU_BICGSTAB_IR32, hA, hB, hX, tol=args.tol)
        assert r["status"] == 0, r
    e2e_ms = max_over_ranks(1000.0 * (time.perf_counter() - t0) / args.steps)
    barrier()
    # ---- the same with pageable host buffers: plain numpy arrays, like the
    # std::vector storage the C++ drop-in hands over
    pA, pB, pX = s.value.copy(), s.b.copy(), np.zeros(s.n)
    for _ in range(args.warmup):
        pX[:] = 0.0
        ctx.solve(ocsl.ILU_BICGSTAB_IR32, pA, pB, pX, tol=args.tol)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        pX[:] = 0.0
        r = ctx.solve(ocsl.ILU_BICGSTAB_IR32, pA, pB, pX, tol=args.tol)
        assert r["status"] == 0, r
    e2e_pageable_ms = max_over_ranks(1000.0 * (time.perf_counter() - t0) / args.steps)
    barrier()

    # ---- roofline of the dominant kernel in the headline timed region
    peak, peak_kind = load_peaks()
    structured = ctx.sweep_info()["kind"] in (2, 3)
    algo = algorithmic_bytes(s.n, s.nnz_real, nnz_l, nnz_u, structured)
    per_cat = {k: {"ms_total": v[0], "launches": v[1]} for k, v in prof_ir.items() if v[1]}
    total_ms = sum(v["ms_total"] for k, v in per_cat.items())
    dom = max((k for k in per_cat if k in algo), key=lambda k: per_cat[k]["ms_total"])
    launches = per_cat[dom]["launches"]
    avg_ms = per_cat[dom]["ms_total"] / launches
    achieved = algo[dom] / (avg_ms * 1e-3) / 1e9
    traffic = load_traffic().get(dom) if structured else None
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, burst copy)",
                "unit": "GB/s", "frac": achieved / peak, "traffic": traffic,
                "algorithmic_bytes_per_launch": algo[dom], "avg_launch_ms": avg_ms,
                "share_of_kernel_time": per_cat[dom]["ms_total"] / total_ms if total_ms else None,
                "measured": "per-launch CUDA events on the library stream over a second timed "
                            "pass of the same solves (ms_per_step of that pass: "
                            f"{ms_ir_prof:.3f})"}
    kernel_gbs = {}
    for prof in (prof_ir, prof_64):
        for k, (msk, cnt) in prof.items():
            if cnt and k in algo:
                kernel_gbs[k] = round(algo[k] / (msk / cnt * 1e-3) / 1e9, 1)
    # every kernel of the library in the timed solves (the profiled pass runs
    # the same launch sequence, without graph replay)
    gpu_launches = sum(v["launches"] for v in per_cat.values())

    # ---- the reference's CPU-runnable case (1000-cell shock tube) end to end
    simple = simple_iteration(torch, dev) if rank == 0 else None
    if rank == 0 and args.flow_size > 0:
        simple["at_scale"] = simple_iteration_at_scale(args.flow_size, args.flow_inner)

    # ---- CPU baseline: reference algorithm, bounded sample, rank 0
    cpu = None
    if rank == 0:
        threads = os.cpu_count() or 1
        rate, calls, el = cpu_reference_rate(s, args.cpu_seconds, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{calls} reference ILU_BICGSTAB_solve() calls (ILU + 3 fixed "
                         f"iterations; the reference cannot reach 1e-10) on this system in "
                         f"{el:.1f} s, OpenMP port of cmatrix_solver.cpp:682-762"}

    if rank == 0:
        it_in = [i for i, _, _ in its_ir]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_ir,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded)",
            "config": workload_config(args.size, s.n, s.nnz, s.nnz_real),
            "e2e": {"value": world * 1000.0 / e2e_ms, "unit": UNIT,
                    "h2d_bytes_per_step": int(8 * (s.nnz + 2 * s.n)),
                    "d2h_bytes_per_step": int(8 * s.n)},
            "e2e_pageable": {"value": world * 1000.0 / e2e_pageable_ms, "unit": UNIT,
                             "h2d_bytes_per_step": int(8 * (s.nnz + 2 * s.n)),
                             "d2h_bytes_per_step": int(8 * s.n),
                             "host_buffers": "pageable (numpy), as the C++ drop-in passes "
                                             "std::vector storage"},
            "gpu_launches": gpu_launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "clocks": clk,
            "fp64_solves_per_s": world * 1000.0 / ms_64,
            "ir32_speedup_vs_fp64": ms_64 / ms_ir,
            "reference_solve_calls_per_s_gpu": world * 1000.0 / ms_ref,
            "iterations": {"ir32_inner": it_in[-1], "ir32_outer": its_ir[-1][1],
                           "fp64": its_64[-1][0]},
            "relres": {"ir32": its_ir[-1][2], "fp64": its_64[-1][2]},
            "spmv_gbs": {k: v for k, v in kernel_gbs.items() if k.startswith("spmv")},
            "kernel_gbs": kernel_gbs,
            "kernel_ms": {k: round(v["ms_total"] / args.steps, 4) for k, v in per_cat.items()},
            "setup_s": {"generate": round(t_gen, 2), "set_pattern": round(t_pat, 3),
                        "autotune": round(t_tune, 3)},
            "sweep_kernel": dict(ctx.sweep_info(), autotuned_pair_us=round(tune["sweep_us"], 1),
                                 autotuned_pair_us_f64=round(tune64["sweep_us"], 1)),
            "multicolour_ordering": multicolour,
            "simple_iteration": simple,
        }
        print(json.dumps(line))
    ctx.close()
    group.close()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
