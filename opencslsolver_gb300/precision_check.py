"""Mixed-precision check on one workload: the FP32-refined ILU-BiCGSTAB and
the plain FP64 one, both to 1e-10 relative residual from x0 = 0, against an
FP64 solution run to 1e-13 (the FP64 tolerance-mode solver is the oracle's
algorithm bit for bit -- tests/test_gpu_solvers.py -- so at full size it
stands in for the CPU oracle, which would take minutes).

    python -m opencslsolver_gb300.precision_check --tet 64        # 64^3 x 6 tets, Peclet <= 50
    python -m opencslsolver_gb300.precision_check --hex 128       # 128^3 hex, Peclet <= 10

Prints one JSON line: solves/s (CUDA-event time of the solve, best of
--reps), iterations, true relative residuals and the relative solution error
||x - x_ref||_2 / ||x_ref||_2 of each method.
"""
from __future__ import annotations

import argparse
import json
import sys


def main(argv=None):
    ap = argparse.ArgumentParser()
    g = ap.add_mutually_exclusive_group()
    g.add_argument("--tet", type=int, default=None)
    g.add_argument("--hex", type=int, default=None)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)

    import torch

    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import workloads as W

    if a.hex is not None:
        s = W.hex_pprime(a.hex, peclet=10.0)
    else:
        s = W.tet_pprime(a.tet if a.tet is not None else 64, peclet=50.0)
    ctx = ocsl.Context(0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch.from_numpy(s.value).cuda()
    B = torch.from_numpy(s.b).cuda()

    def solve(method, tol):
        best, X = None, None
        for _ in range(a.reps):
            X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
            r = ctx.solve_device(method, A, B, X, tol=tol)
            if r["status"] != 0:
                raise RuntimeError(f"{method}: {r}")
            best = r if best is None or r["solve_ms"] < best["solve_ms"] else best
        return X, best

    def relres(X):
        y = torch.empty_like(X)
        ctx.gemv_device(A, X, y, mode=1, z=B)
        return float(torch.linalg.norm(y) / torch.linalg.norm(B))

    x_ref, r_ref = solve(ocsl.ILU_BICGSTAB, 1e-13)
    out = {"workload": s.name, "n": s.n, "nnz_real": s.nnz_real,
           "sweep_kernel": ctx.sweep_info()["kind"],
           "reference_solution": {"method": "FP64 ILU-BiCGSTAB to 1e-13",
                                  "relres": relres(x_ref), "iterations": r_ref["iterations"]}}
    for name, method in (("fp32_refined", ocsl.ILU_BICGSTAB_IR32), ("fp64", ocsl.ILU_BICGSTAB)):
        X, r = solve(method, 1e-10)
        out[name] = {"solves_per_s": round(1000.0 / r["solve_ms"], 2),
                     "solve_ms": round(r["solve_ms"], 3), "iterations": r["iterations"],
                     "outer_iterations": r["outer_iterations"], "relres": relres(X),
                     "error_vs_fp64_reference": float(torch.linalg.norm(X - x_ref) /
                                                      torch.linalg.norm(x_ref))}
    out["speedup_fp32_refined_vs_fp64"] = round(out["fp64"]["solve_ms"] /
                                                out["fp32_refined"]["solve_ms"], 3)
    print(json.dumps(out))
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
