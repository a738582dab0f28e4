"""Time the GPU face-loop assembly on a hex flow state (the target of ncu
captures of assemble_kernel, too).

    python -m opencslsolver_gb300.assembly_bench --size 128 [--reps 20]

Assembles the pressure-correction, one momentum component and the enthalpy
equation of the seeded hex-box flow state (workloads.hex_flow_state) and
prints one JSON line: CUDA-event time per assembly and the algorithmic bytes
each one must move -- per cell its incidence entries (face index and CSR slot,
8 B per face side), the face fields it reads (geo_aver, mdot, and per
equation density / Qy or ksi_A: 8 B each per face side), the neighbour cell
fields (8 B per face side per field) and its own fields, plus the outputs
(values 8 B per stored entry, b and x0).
"""
from __future__ import annotations

import argparse
import json
import sys


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--reps", type=int, default=20)
    a = ap.parse_args(argv)

    import numpy as np
    import torch

    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import _abi
    from opencslsolver_gb300 import workloads as W

    f = W.hex_flow_state(a.size)
    ctx = ocsl.Context(0)
    ctx.set_pattern(f.row_ptr, f.column_index)
    ctx.set_faces(f.left, f.right, f.bc_left)
    st = {}
    for k, v in f.state.items():
        dt = torch.int32 if k in _abi.INT_FIELDS else torch.float64
        st[k] = torch.as_tensor(np.ascontiguousarray(v)).to(device="cuda", dtype=dt)
    n, nnz = f.n, f.column_index.size
    value = torch.empty(nnz, dtype=torch.float64, device="cuda")
    b, x0 = (torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(2))
    sides = 2 * f.left.size
    # bytes per equation: incidence (8 / side) + face fields + neighbour fields + own fields + outputs
    per_eq = {
        "pressure": (6, 3, 6),   # face: geo, mdot, density, qy (+stress none) ; nbr: T, p'; own: vol, dt, rho, rho_last, T, p'
        "momentum_x": (2, 1, 6),  # face: geo, mdot; nbr: u; own: vol, dt, rho, rho_last, u_last, grad p
        "enthalpy": (3, 2, 7),    # face: geo, mdot, ksi; nbr: h, T; own: vol, dt, rho, rho_last, h_last, p, p_last
    }
    out = {"workload": f.name, "n": n, "faces": int(f.left.size), "bc_faces": int(f.bc_left.size)}
    for name, eqn, dim in (("pressure", 1, 0), ("momentum_x", 0, 0), ("enthalpy", 2, 0)):
        eq = dict(f.eq, equation=eqn, dimension=dim)
        ctx.assemble_device(eq, st, value, b, x0)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.reps):
            ctx.assemble_device(eq, st, value, b, x0)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / a.reps
        fface, fnbr, fown = per_eq[name]
        algo = 8 * sides + 8 * fface * sides + 8 * fnbr * sides + 8 * fown * n + 8 * nnz + 16 * n
        out[name] = {"ms": round(ms, 4), "algorithmic_bytes": int(algo),
                     "gb_per_s": round(algo / (ms * 1e-3) / 1e9, 1)}
    print(json.dumps(out))
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
