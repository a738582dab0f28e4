"""The whole SIMPLE inner iteration at scale, from a mesh file.

    python -m opencslsolver_gb300.flow_bench --size 128 --inner 10

A seeded N^3 jittered hex box of the unit cube written as SU2
(``workloads.write_su2_box``), read by the library (``read_su2``: the
reference's face numbering and finite-volume metrics in O(cells + faces)),
its matrix pattern built from the faces (``build_pattern``), the initial
state of CFlow_solver::initialize (``flow.initial_state``: a 3D viscous channel,
velocity inlet (20, 3, 2) m/s at 300 K, no-slip walls, pressure outlet, 1e5 Pa,
transient dt 2e-6 s, blended convection), then ``--inner`` device inner
iterations with each solver choice, the reference's (one CUDA graph per
iteration), the FP64 tolerance mode and the FP32-inner / FP64-refined mode,
the last two also through the multicolour ordering (ocsl_set_ordering).
With ``--vtk`` the state after the first choice's iterations is written from
device memory as the reference's solution.vtk / solution_BC.vtk
(``Mesh.write_vtk``, ocsl_vtk_write), timed.
Prints one JSON object (``bench.py`` times the CPU restatement beside it).
"""
from __future__ import annotations

import argparse
import json
import os
import tempfile
import time

CONFIG = dict(initial={"pressure": 1e5, "temperature": 300.0, "velocity": (20, 0, 0)},
              boundaries=[{"kind": "velocity_inlet", "velocity": (20, 3, 2),
                           "temperature": 300.0, "pressure": 1e5},
                          {"kind": "wall", "wall": "no_slip"},
                          {"kind": "pressure_outlet", "pressure": 1e5}],
              viscous=True, blended=True, transient=True, dt=2e-6)


def box_case(size: int, keep_dir: str | None = None):
    """The N^3 box case: SU2 file -> read_su2 -> build_pattern ->
    initial_state.  Returns (case, set-up facts); the SU2 file stays in
    keep_dir (as box.su2) when given."""
    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import flow as F
    from opencslsolver_gb300 import workloads as W

    info = {"workload": f"{size}^3 jittered hex box from SU2, 3D viscous channel (velocity "
                        "inlet, no-slip walls, pressure outlet), transient"}
    with tempfile.TemporaryDirectory() as tmp:
        d = keep_dir or tmp
        path = os.path.join(d, "box.su2")
        t0 = time.perf_counter()
        W.write_su2_box(path, size, size, size, lengths=(1.0, 1.0, 1.0))
        info["write_su2_s"] = round(time.perf_counter() - t0, 2)
        info["su2_bytes"] = os.path.getsize(path)
        t0 = time.perf_counter()
        mesh = ocsl.read_su2(path)
        info["read_su2_s"] = round(time.perf_counter() - t0, 2)
    t0 = time.perf_counter()
    rp, col = ocsl.build_pattern(mesh["n_cells"], mesh["face_left"], mesh["face_right"],
                                 mesh["bc_left"])
    mesh.update(row_ptr=rp, column_index=col)
    info["build_pattern_s"] = round(time.perf_counter() - t0, 2)
    t0 = time.perf_counter()
    case = F.initial_state(mesh, **CONFIG)
    info["initial_state_s"] = round(time.perf_counter() - t0, 2)
    info.update(cells=int(mesh["n_cells"]), faces=int(mesh["n_faces"]),
                bc_faces=int(mesh["n_bc"]), nnz=int(col.size))
    return case, info


def methods():
    import opencslsolver_gb300 as ocsl

    return {"reference_solvers": (ocsl.BICGSTAB_REF,) * 3,
            "fp64_tolerance": (ocsl.ILU_BICGSTAB,) * 3,
            "fp32_refined": (ocsl.ILU_BICGSTAB_IR32,) * 3}


# solver choices run a second time through the multicolour ordering
MULTICOLOUR = ("fp64_tolerance", "fp32_refined")


def write_vtk(run, su2_path: str, out_dir: str) -> dict:
    """The run's device state as the reference's two VTK files; seconds
    (mesh read, write) and file sizes."""
    import torch

    import opencslsolver_gb300 as ocsl

    st, ar, eq = run.state, run.arrays, run.case["eq"]
    t0 = time.perf_counter()
    mesh = ocsl.Mesh(su2_path)
    t1 = time.perf_counter()
    cells, bc = os.path.join(out_dir, "solution.vtk"), os.path.join(out_dir, "solution_BC.vtk")
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    mesh.write_vtk(cells, bc, density=st["density_c"], pressure=st["pressure"],
                   temperature=st["temperature"], mach=ar["mach"], velocity=st["velocity"],
                   pressure_grad=st["pressure_grad"], bc_type=st["bc_type"],
                   bc_wall=st["bc_wall"], viscous=bool(eq["viscous"]),
                   sutherland=eq["sutherland"])
    t3 = time.perf_counter()
    mesh.close()
    return {"mesh_read_s": round(t1 - t0, 2), "write_s": round(t3 - t2, 3),
            "bytes": os.path.getsize(cells) + os.path.getsize(bc),
            "threads": os.cpu_count()}


def time_gpu(case: dict, inner: int, device: int = 0, only=None, vtk_from=None) -> dict:
    """ms per inner iteration for every solver choice (two untimed calls
    first: allocation, then the graph capture of the reference's solvers);
    `only`: the one choice to run (a key of the result); vtk_from: the SU2
    file, to write the first choice's final state as VTK."""
    import copy

    import numpy as np
    import torch

    import opencslsolver_gb300 as ocsl
    from opencslsolver_gb300 import flow as F

    ctx = ocsl.Context(device)
    out = {}
    runs = [(name, m, "natural") for name, m in methods().items()]
    runs += [(name + "_multicolour", methods()[name], "multicolour") for name in MULTICOLOUR]
    if only is not None:
        runs = [r for r in runs if r[0] == only]
        if not runs:
            raise ValueError(f"unknown solver choice {only!r}")
    try:
        for name, m, ordering in runs:
            ctx.set_ordering(ordering)
            run = F.FlowRun(ctx, copy.deepcopy(case))
            run.iterate(m)
            run.iterate(m)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(inner):
                rep = run.iterate(m)
            torch.cuda.synchronize()
            ms = 1000.0 * (time.perf_counter() - t0) / inner
            f = run.fields()
            out[name] = {"ms_per_inner_iteration": round(ms, 3), "status": rep["status"],
                         "solve_iterations_last": rep["iterations"],
                         "residuals_last": [float(v) for v in rep["residual"]],
                         "finite": bool(all(np.all(np.isfinite(v)) for v in f.values()))}
            if vtk_from and "vtk" not in out:
                with tempfile.TemporaryDirectory() as d:
                    out["vtk"] = write_vtk(run, vtk_from, d)
            del run
            torch.cuda.empty_cache()
    finally:
        ctx.close()
    return out


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--size", type=int, default=128)
    ap.add_argument("--inner", type=int, default=10)
    ap.add_argument("--only", default=None,
                    help="run one solver choice (e.g. fp32_refined_multicolour)")
    ap.add_argument("--vtk", action="store_true",
                    help="write the first choice's final state as VTK from the device, timed")
    a = ap.parse_args(argv)
    with tempfile.TemporaryDirectory() as d:
        case, info = box_case(a.size, keep_dir=d if a.vtk else None)
        info["gpu"] = time_gpu(case, a.inner, only=a.only,
                               vtk_from=os.path.join(d, "box.su2") if a.vtk else None)
    print(json.dumps(info))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
