"""Run a few solves of one configuration: the target of `ncu` captures.

    python -m opencslsolver_gb300.profile_case --size 128 --method ilu_bicgstab_ir32 --solves 2

Generates the seeded hex p' system of the given size, uploads it once and runs
``--solves`` solves on cuda:0 (no timing, no checks beyond the status), so a
profiler can pick individual kernel launches out of a realistic solve.
"""
from __future__ import annotations

import argparse
import sys

import numpy as np


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--method", default="ilu_bicgstab_ir32")
    ap.add_argument("--solves", type=int, default=2)
    ap.add_argument("--sweep-kernel", type=int, default=0)
    ap.add_argument("--tet", action="store_true", help="tetrahedral (6 per hex) system")
    ap.add_argument("--dims", type=int, nargs=3, default=None, help="hex box nx ny nz")
    ap.add_argument("--tiles", type=int, nargs=2, default=(0, 0), help="structured sweep tile")
    ap.add_argument("--cluster", type=int, nargs=2, default=(1, 1),
                    help="structured sweep tiles per thread-block cluster")
    ap.add_argument("--inner-tol", type=float, default=None, help="IR32 inner tolerance")
    ap.add_argument("--ordering", default="natural", choices=["natural", "multicolour"],
                    help="row ordering of the tolerance-mode solves")
    ap.add_argument("--profile", action="store_true",
                    help="print CUDA-event time per launch by kernel category (last solve)")
    a = ap.parse_args(argv)

    import torch

    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import workloads as W

    if a.tet:
        s = W.tet_pprime(a.size, peclet=50.0)
    elif a.dims:
        s = W.hex_pprime(*a.dims, peclet=10.0)
    else:
        s = W.hex_pprime(a.size, peclet=10.0)
    ctx = ocsl.Context(0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_sweep_kernel(a.sweep_kernel, *a.tiles)
    ctx.set_sweep_cluster(*a.cluster)
    ctx.set_ordering(a.ordering)
    A = torch.from_numpy(s.value).cuda()
    B = torch.from_numpy(s.b).cuda()
    X = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    for k in range(a.solves):
        if a.profile and k == a.solves - 1:
            ctx.profile(True)
            ctx.profile_read()
        X.zero_()
        opts = {} if a.inner_tol is None else {"inner_tol": a.inner_tol}
        r = ctx.solve_device(a.method, A, B, X, **opts)
        if r["status"] != 0:
            print("solve failed", r, file=sys.stderr)
            return 1
    torch.cuda.synchronize()
    if a.profile:
        for name, (ms, count) in ctx.profile_read().items():
            if count:
                print(f"{name:14s} {count:5d} launches  {1000.0 * ms / count:9.1f} us/launch")
    print(f"{s.name}: {a.solves} x {a.method}: {r} sweep {ctx.sweep_info()}")
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
