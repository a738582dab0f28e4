"""Throughput of the batching workload: 64 hex boxes (cells log-uniform in
[1e4, 5e5], aspect U[1, 4] per axis), each with one p' system (1 right-hand
side) and one momentum system (3 right-hand sides sharing the matrix) --
256 solves to 1e-10 relative residual from x0 = 0.

    python -m opencslsolver_gb300.batch_bench [--count 64] [--workers 16]

Prints one JSON line: wall time of the whole batch solved concurrently
(ocsl_batch_solve_device, FP32-refined and plain FP64; FP32-refined also in
the one-graph mode, ocsl_batch_set_graph: one graph launch for all 256 solves
with every loop on the device, replayed after its first call) and of the same 256
plain-FP64 solves one after the other on one stream (the same batch object
with one worker), with every solve's true relative residual checked on the
device.  Inputs are resident on the device before the clock starts.
"""
from __future__ import annotations

import argparse
import json
import sys
import time


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=64)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--min-cells", type=int, default=10_000)
    ap.add_argument("--max-cells", type=int, default=500_000)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args(argv)

    import numpy as np
    import torch

    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import workloads as W

    t0 = time.perf_counter()
    systems = W.batch_systems(a.count, min_cells=a.min_cells, max_cells=a.max_cells)
    gen_s = time.perf_counter() - t0
    spec = [(b.system.row_ptr, b.system.column_index, b.rhs.shape[0]) for b in systems]
    vals = [torch.from_numpy(b.system.value).cuda() for b in systems]
    Bs = [torch.from_numpy(np.ascontiguousarray(b.rhs)).cuda() for b in systems]
    Xs = [torch.zeros_like(B) for B in Bs]

    def run(batch, method):
        best, last = None, None
        for _ in range(a.reps):
            for X in Xs:
                X.zero_()
            torch.cuda.synchronize()
            t = time.perf_counter()
            st, res = batch.solve_device(method, vals, Bs, Xs, tol=1e-10)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t
            if st != 0:
                raise RuntimeError(f"batch status {st}")
            best = dt if best is None else min(best, dt)
            last = res
        return best, last

    def max_relres():
        ctx = ocsl.Context(0)
        worst = 0.0
        for b, v, B, X in zip(systems, vals, Bs, Xs):
            ctx.set_pattern(b.system.row_ptr, b.system.column_index)
            for r in range(B.shape[0]):
                y = torch.empty_like(B[r])
                ctx.gemv_device(v, X[r].contiguous(), y, mode=1, z=B[r].contiguous())
                worst = max(worst, float(torch.linalg.norm(y) / torch.linalg.norm(B[r])))
        ctx.close()
        return worst

    t0 = time.perf_counter()
    conc = ocsl.Batch(spec, workers=a.workers)
    setup_s = time.perf_counter() - t0
    run(conc, ocsl.ILU_BICGSTAB_IR32)  # warm-up
    t_ir32, res_ir32 = run(conc, ocsl.ILU_BICGSTAB_IR32)
    rr_ir32 = max_relres()
    t_fp64, res_fp64 = run(conc, ocsl.ILU_BICGSTAB)
    rr_fp64 = max_relres()
    conc.set_graph(True)
    t0 = time.perf_counter()
    for X in Xs:  # the first call captures and instantiates the graph
        X.zero_()
    st_g, _ = conc.solve_device(ocsl.ILU_BICGSTAB_IR32, vals, Bs, Xs, tol=1e-10)
    torch.cuda.synchronize()
    t_capture = time.perf_counter() - t0
    if st_g != 0:
        raise RuntimeError(f"graph batch status {st_g}")
    t_graph, res_graph = run(conc, ocsl.ILU_BICGSTAB_IR32)
    rr_graph = max_relres()
    same = all(r1["iterations"] == r2["iterations"] for r1, r2 in zip(res_ir32, res_graph))
    conc.close()
    seq = ocsl.Batch(spec, workers=1)
    run(seq, ocsl.ILU_BICGSTAB)  # warm-up
    t_seq, _ = run(seq, ocsl.ILU_BICGSTAB)
    seq.close()
    cells = [b.system.n for b in systems[::2]]
    solves = sum(B.shape[0] for B in Bs)
    print(json.dumps({
        "workload": f"{a.count} hex boxes, cells log-uniform [{a.min_cells}, {a.max_cells}], "
                    "aspect U[1,4]; p' (1 rhs) + momentum (3 rhs) each",
        "boxes": a.count, "solves": solves, "cells_total": int(sum(cells)),
        "workers": a.workers,
        "batched_ir32_s": round(t_ir32, 4), "batched_fp64_s": round(t_fp64, 4),
        "sequential_fp64_s": round(t_seq, 4),
        "speedup_batched_ir32_vs_sequential_fp64": round(t_seq / t_ir32, 2),
        "speedup_batched_fp64_vs_sequential_fp64": round(t_seq / t_fp64, 2),
        "solves_per_s_batched_ir32": round(solves / t_ir32, 1),
        "graph_ir32_s": round(t_graph, 4),
        "graph_first_call_s": round(t_capture, 4),
        "solves_per_s_graph_ir32": round(solves / t_graph, 1),
        "graph_iterations_equal_host_batch": same,
        "max_true_relres": {"ir32": rr_ir32, "fp64": rr_fp64, "ir32_graph": rr_graph},
        "iterations_total": {"ir32": int(sum(r["iterations"] for r in res_ir32)),
                             "fp64": int(sum(r["iterations"] for r in res_fp64))},
        "setup_s": {"generate": round(gen_s, 1), "batch_create": round(setup_s, 1)},
    }))
    return 0


if __name__ == "__main__":
    sys.exit(main())
