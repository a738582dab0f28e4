"""Generate the golden fixtures of tests/golden/ from the reference itself.

Run in a container where the reference's sources are present:

    python tests/golden/make_golden.py [--reference <reference source dir>]

(default: OCSL_REFERENCE_DIR, else a checkout named "reference" beside this
repository).

It builds the reference from its own sources (oracle/Makefile, target `ref`),
then writes:

* kat_tridiag10.npz -- the reference's own solver unit-test system
  (cmatrix_solver_supply.h:29-114: 10x10 tridiagonal [1, 5, 1], b = 2,
  x0 = 1), with the residual and x returned by the reference's CG_solve and
  ILU_BICGSTAB_solve (the latter with M prepared as cfvm.cpp:96-97 does; the
  unit test as written never prepares it and crashes);
* shocktube_calls.npz -- linear systems captured from the reference's SIMPLE
  loop on the 1000-cell shock tube (momentum solves with CG, p' and enthalpy
  with ILU-BiCGSTAB): values, b, x0, the reference's x and residual, and the
  final fields (p, u, T, rho) at full precision;
* small_systems.npz -- seeded small systems in the reference layout with the
  reference's gemv, ILU_decompose, ILU_forsub/backsub, CG_solve and
  ILU_BICGSTAB_solve outputs;
* flow_<case>.npz -- the reference's SIMPLE loop, recorded by
  oracle/ref_flow.cpp one inner iteration at a time, on the shock tube
  (200 steps x 5 inner iterations), the 200-cell viscous channel (100 x 3),
  the 200-cell viscous steady case (60 x 1) and a 3D viscous channel on a
  240-cell jittered hex mesh read from an SU2 file (40 x 3) of FLOW_CASES: the setup
  (mesh metrics, fluid constants, switches, initial state; keys setup__*);
  for three recorded inner iterations of the run with every equation through
  ILU_BICGSTAB_solve, the state before the iteration (start_<tag>__*, with
  endstep_<tag> when the step's update_timestep comes first; the first
  starts from the setup), the five assembled systems and the reference's
  solutions (value_<tag>, b_<tag>, x0_<tag>, x_<tag>), the under-relaxation
  in force (relax_<tag>) and the state after it (post_<tag>__*); the final
  state of that run (final_bicg__*) and, for the shock tube, of the run with
  the momentum equations through CG_solve (final_cg__*);
* mesh_<cells>.npz -- the reference's finite-volume arrays (face numbering,
  metrics, cell volumes) and matrix pattern for a 5 x 4 x 3 jittered box of
  hexahedra, tetrahedra or wedges that it read from the SU2 file
  workloads.write_su2_box writes;
* vtk_<cells>.npz -- the reference's own VTK output (solution.vtk and
  solution_BC.vtk, as bytes) after a short run of the 3D viscous channel on a
  jittered box of hexahedra, tetrahedra or wedges read from an SU2 file, with
  the final state and fluid constants it was written from; vtk_heat.npz the
  same for a heat-conduction run on a hex box (fixed temperatures at the
  inlet and outlet markers, adiabatic walls);
* assembly_<case>.npz -- the inputs (cell / face state) and outputs (matrix
  values, b, x0, ap_vec, total_mdot) of the reference's face-loop assembly,
  recorded by oracle/ref_assembly.cpp right before the 5 solve calls of one
  SIMPLE inner iteration, for three cases: the 1000-cell shock tube
  (inviscid, blended, transient, slip walls), a 200-cell viscous channel
  (upwind, transient, velocity inlet, no-slip walls, pressure outlet) and a
  200-cell steady case (viscous, blended, implicit under-relaxation,
  supersonic inlet, slip walls, outlet), and three time steps of a 100-cell
  heat-conduction run (fixed temperatures at the ends, adiabatic sides).
  Mesh arrays are stored once per case, state and outputs per call with the
  prefix c<k>_.

All reference calls use one OpenMP thread (deterministic reduction order).
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from opencslsolver_gb300 import workloads as W  # noqa: E402
from oracle import oracle as orc  # noqa: E402

# Recorded solve calls: (step, inner iteration) of the 200-step, 5-inner run.
SHOCKTUBE_RECORD = ["0:0", "0:4", "100:2", "199:4"]


def tridiag10():
    n = 10
    rp, col, val = [0], [], []
    for i in range(n):
        for j in (i - 1, i, i + 1):
            if 0 <= j < n:
                col.append(j)
                val.append(5.0 if j == i else 1.0)
        rp.append(len(col))
    return (np.array(rp, np.uint64), np.array(col, np.uint64), np.array(val), np.full(n, 2.0),
            np.ones(n))


def make_kat(ref, out):
    rp, col, val, b, x0 = tridiag10()
    xc, rc = ref.cg_solve(rp, col, val, b, x0)
    xb, rb = ref.bicgstab_solve(rp, col, val, b, x0)
    np.savez_compressed(out, row_ptr=rp, column_index=col, value=val, b=b, x0=x0, cg_x=xc,
                        cg_res=rc, bicg_x=xb, bicg_res=rb)


def make_shocktube(out):
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([orc.REF_SHOCKTUBE, d, "1", "200", "5", *SHOCKTUBE_RECORD], cwd=d,
                       check=True, stdout=subprocess.DEVNULL)
        raw = open(os.path.join(d, "pattern.bin"), "rb").read()
        n, nnz = np.frombuffer(raw[:16], np.uint64).astype(int)
        rp = np.frombuffer(raw[16:16 + 8 * (n + 1)], np.uint64)
        col = np.frombuffer(raw[16 + 8 * (n + 1):], np.uint64)
        calls = sorted(f for f in os.listdir(d) if f.startswith("call_"))
        meta, res, vals, bs, x0s, xs = [], [], [], [], [], []
        for f in calls:
            buf = open(os.path.join(d, f), "rb").read()
            hdr = np.frombuffer(buf[:16], np.int32)
            nn, nz = np.frombuffer(buf[16:32], np.uint64).astype(int)
            r = np.frombuffer(buf[32:40], np.float64)[0]
            off = 40
            v = np.frombuffer(buf[off:off + 8 * nz], np.float64); off += 8 * nz
            b = np.frombuffer(buf[off:off + 8 * nn], np.float64); off += 8 * nn
            x0 = np.frombuffer(buf[off:off + 8 * nn], np.float64); off += 8 * nn
            x = np.frombuffer(buf[off:off + 8 * nn], np.float64); off += 8 * nn
            xcopy = np.frombuffer(buf[off:off + 8 * nn], np.float64)
            assert np.array_equal(x, xcopy), f"{f}: reference not deterministic"
            meta.append(np.concatenate([hdr, [int(f[5:10])]]))
            res.append(r); vals.append(v); bs.append(b); x0s.append(x0); xs.append(x)
        fields = np.loadtxt(os.path.join(d, "fields.txt"))
    np.savez_compressed(out, row_ptr=rp, column_index=col, meta=np.array(meta, np.int32),
                        residual=np.array(res), value=np.array(vals), b=np.array(bs),
                        x0=np.array(x0s), x=np.array(xs), fields=fields)


def small_cases():
    return [W.hex_pprime(6, peclet=10.0), W.hex_pprime(6, 5, 4, peclet=0.0),
            W.tet_pprime(3, peclet=50.0), W.random_rows_system(200, 9, seed=11),
            W.System(*W.pattern_1d(50), np.zeros(0), np.zeros(0), "oned50")]


def make_small(ref, out):
    arrays = {}
    rng = np.random.default_rng(5)
    for k, s in enumerate(small_cases()):
        if s.name == "oned50":  # 1D pattern with diagonally dominant values
            rp, col = s.row_ptr, s.column_index
            val = np.where(col == W.PHANTOM, 0.0, -1.0)
            rows = np.repeat(np.arange(s.n), np.diff(rp.astype(np.int64)))
            val[(col == rows.astype(np.uint64))] = 2.5
            s = W.System(rp, col, val, rng.uniform(-1, 1, s.n), "oned50")
        rp, col, val, b = s.row_ptr, s.column_index, s.value, s.b
        x0 = rng.uniform(-1, 1, s.n) * 0.1
        z = rng.uniform(-1, 1, s.n)
        xin = rng.uniform(-1, 1, s.n)
        p = f"c{k}_"
        arrays[p + "name"] = np.array(s.name)
        arrays[p + "row_ptr"], arrays[p + "column_index"] = rp, col
        arrays[p + "value"], arrays[p + "b"], arrays[p + "x0"] = val, b, x0
        arrays[p + "z"], arrays[p + "xin"] = z, xin
        arrays[p + "gemv0"] = ref.gemv(rp, col, val, 1.0, xin)
        arrays[p + "gemv1"] = ref.gemv(rp, col, val, -1.0, xin, 1.0, z)
        arrays[p + "gemv2"] = ref.gemv(rp, col, val, -0.37, xin, 1.0, z)
        M = ref.ilu_decompose(rp, col, val)
        arrays[p + "ilu"] = M
        arrays[p + "forsub"] = ref.forsub(rp, col, M, z)
        arrays[p + "backsub"] = ref.backsub(rp, col, M, z)
        xc, rc = ref.cg_solve(rp, col, val, b, x0)
        xb, rb = ref.bicgstab_solve(rp, col, val, b, x0)
        arrays[p + "cg_x"], arrays[p + "cg_res"] = xc, rc
        arrays[p + "bicg_x"], arrays[p + "bicg_res"] = xb, rb
    arrays["count"] = np.array(len(small_cases()))
    np.savez_compressed(out, **arrays)


# (case, first recorded solve call, calls): the last inner iteration of each
# flow run (5 equations), three time steps of the heat run.
ASSEMBLY_CASES = [("shocktube", 25, 5), ("channel", 25, 5), ("steady", 15, 5), ("heat", 3, 3)]
MESH_KEYS = ("face_left", "face_right", "face_geo_aver", "face_ksi_A", "bc_left", "bc_area",
             "bc_area_vector", "bc_perp_dist", "bc_ksi_A", "cell_volume", "row_ptr",
             "column_index", "bc_type", "bc_wall", "bc_thermal")


def read_named_arrays(path):
    """The dump format of oracle/ref_assembly.cpp."""
    kinds = {"d": "<f8", "i": "<i4", "u": "<u8"}
    data = open(path, "rb").read()
    out, o = {}, 0
    while o < len(data):
        ln = int(np.frombuffer(data, "<u4", 1, o)[0]); o += 4
        name = data[o:o + ln].decode(); o += ln
        dt = np.dtype(kinds[chr(data[o])]); o += 1
        cnt = int(np.frombuffer(data, "<u8", 1, o)[0]); o += 8
        out[name] = np.frombuffer(data, dt, cnt, o).copy(); o += dt.itemsize * cnt
    return out


def make_assembly(out_dir):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_assembly")
    for case, first, count in ASSEMBLY_CASES:
        arrays = {}
        with tempfile.TemporaryDirectory() as d:
            subprocess.run([exe, d, case, str(first), str(count)], cwd=d, check=True,
                           stdout=subprocess.DEVNULL)
            calls = sorted(f for f in os.listdir(d) if f.startswith("call_"))
            assert len(calls) == count, calls
            for k, f in enumerate(calls):
                z = read_named_arrays(os.path.join(d, f))
                for key, v in z.items():
                    if key in MESH_KEYS:
                        if key in arrays:
                            assert np.array_equal(arrays[key], v), key
                        arrays[key] = v
                    else:
                        arrays[f"c{k}_{key}"] = v
        arrays["count"] = np.array(count)
        np.savez_compressed(os.path.join(out_dir, f"assembly_{case}.npz"), **arrays)


# The flow fixtures: run length, recorded inner iterations (tag "s_i" =
# step s, inner iteration i) with the record they start from ("setup" = the
# initial state; a start from the previous step's last inner iteration needs
# that step's update_timestep applied first), and whether the run with CG for
# the momentum equations is recorded too.
FLOW_CASES = {
    "shocktube": {"steps": 200, "inner": 5, "cg": True,
                  "iterations": [("setup", "0_0"), ("post_0_0", "0_1"), ("post_57_1", "57_2")]},
    "channel": {"steps": 100, "inner": 3, "cg": False,
                "iterations": [("setup", "0_0"), ("post_0_0", "0_1"), ("post_40_0", "40_1")]},
    "steady": {"steps": 60, "inner": 1, "cg": False,
               "iterations": [("setup", "0_0"), ("post_0_0", "1_0"), ("post_9_0", "10_0")]},
    # 3D viscous channel on a 10 x 6 x 4 jittered hex mesh the reference reads
    # from an SU2 file (workloads.write_su2_box with BOX3D_MESH)
    "box3d": {"steps": 40, "inner": 3, "cg": False,
              "iterations": [("setup", "0_0"), ("post_0_0", "0_1"), ("post_20_0", "20_1")]},
}
BOX3D_MESH = {"nx": 10, "ny": 6, "nz": 4, "lengths": (1.0, 0.2, 0.1), "jitter": 0.1}


def make_flow(out_dir, case):
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_flow")
    spec = FLOW_CASES[case]
    steps, inner = str(spec["steps"]), str(spec["inner"])
    arrays = {"run": np.array([spec["steps"], spec["inner"]])}
    starts = [st for st, _ in spec["iterations"] if st != "setup"]
    tags = [tag for _, tag in spec["iterations"]]
    want = sorted({t.replace("_", ":") for t in tags} |
                  {st[len("post_"):].replace("_", ":") for st in starts})
    with tempfile.TemporaryDirectory() as d:
        arg = case
        if case == "box3d":
            mesh = os.path.join(d, "box3d.su2")
            m = dict(BOX3D_MESH)
            W.write_su2_box(mesh, m.pop("nx"), m.pop("ny"), m.pop("nz"), **m)
            arg = f"box3d={mesh}"
            arrays["mesh"] = np.array([BOX3D_MESH["nx"], BOX3D_MESH["ny"], BOX3D_MESH["nz"]])
        subprocess.run([exe, d, arg, "bicg", steps, inner] + want, cwd=d, check=True,
                       stdout=subprocess.DEVNULL)
        rec = lambda name: read_named_arrays(os.path.join(d, name + ".bin"))  # noqa: E731
        for k, v in rec("setup").items():
            arrays[f"setup__{k}"] = v
        for start, tag in spec["iterations"]:
            if start != "setup":
                for k, v in rec(start).items():
                    arrays[f"start_{tag}__{k}"] = v
                s0, i0 = (int(x) for x in tag.split("_"))
                arrays[f"endstep_{tag}"] = np.array(int(i0 == 0 and s0 > 0))
            for k, v in rec(f"post_{tag}").items():
                arrays[f"post_{tag}__{k}"] = v
            pre = [rec(f"pre_{tag}_{e}") for e in range(5)]
            for key in ("value", "b", "x0", "x"):
                arrays[f"{key}_{tag}"] = np.stack([p[key] for p in pre])
            arrays[f"relax_{tag}"] = pre[0]["implicit_underrelaxation"]
        for k, v in rec("final").items():
            arrays[f"final_bicg__{k}"] = v
    if spec["cg"]:
        with tempfile.TemporaryDirectory() as d:
            subprocess.run([exe, d, case, "cg", steps, inner], cwd=d, check=True,
                           stdout=subprocess.DEVNULL)
            for k, v in read_named_arrays(os.path.join(d, "final.bin")).items():
                arrays[f"final_cg__{k}"] = v
    np.savez_compressed(os.path.join(out_dir, f"flow_{case}.npz"), **arrays)


MESH_KEYS_FVM = ("face_left", "face_right", "face_geo_aver", "face_ksi_A", "face_area_vector",
                 "face_alpha", "face_distance", "face_unit", "bc_left", "bc_area",
                 "bc_area_vector", "bc_alpha", "bc_distance", "bc_unit", "bc_perp_dist",
                 "bc_ksi_A", "cell_volume", "row_ptr", "column_index")


def make_meshes(out_dir):
    """mesh_<cells>.npz: the reference's finite-volume arrays and matrix
    pattern for a 5 x 4 x 3 jittered box of hexahedra, Kuhn tetrahedra or
    wedges read from the SU2 file workloads.write_su2_box writes."""
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_flow")
    for cells in ("hex", "tet", "wedge"):
        with tempfile.TemporaryDirectory() as d:
            mesh = os.path.join(d, "m.su2")
            W.write_su2_box(mesh, 5, 4, 3, cells=cells)
            subprocess.run([exe, d, f"box3d={mesh}", "bicg", "1", "1"], cwd=d, check=True,
                           stdout=subprocess.DEVNULL)
            setup = read_named_arrays(os.path.join(d, "setup.bin"))
        np.savez_compressed(os.path.join(out_dir, f"mesh_{cells}.npz"),
                            **{k: setup[k] for k in MESH_KEYS_FVM})


# The VTK fixtures: the reference's own solution.vtk / solution_BC.vtk
# (Cpost_processing::write_VTK_file / write_boundary_VTK_file) after a short
# run of the 3D viscous channel on a jittered box of hexahedra (the box3d flow
# case), tetrahedra or wedges, with the final state they were written from.
VTK_CASES = {
    "hex": {"mesh": BOX3D_MESH, "cells": "hex", "steps": 40, "inner": 3},
    "tet": {"mesh": {"nx": 5, "ny": 4, "nz": 3, "lengths": (1.0, 0.2, 0.1), "jitter": 0.1},
            "cells": "tet", "steps": 3, "inner": 2},
    "wedge": {"mesh": {"nx": 5, "ny": 4, "nz": 3, "lengths": (1.0, 0.2, 0.1), "jitter": 0.1},
              "cells": "wedge", "steps": 3, "inner": 2},
}


def make_vtk(out_dir):
    """vtk_<cells>.npz: the reference's VTK files (bytes) and the state and
    setup they were written from."""
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_flow")
    for name, spec in VTK_CASES.items():
        with tempfile.TemporaryDirectory() as d:
            mesh = os.path.join(d, "m.su2")
            m = dict(spec["mesh"])
            W.write_su2_box(mesh, m.pop("nx"), m.pop("ny"), m.pop("nz"), cells=spec["cells"], **m)
            subprocess.run([exe, d, f"box3d={mesh}", "bicg", str(spec["steps"]),
                            str(spec["inner"])], cwd=d, check=True, stdout=subprocess.DEVNULL)
            arrays = {f"final__{k}": v
                      for k, v in read_named_arrays(os.path.join(d, "final.bin")).items()}
            setup = read_named_arrays(os.path.join(d, "setup.bin"))
            arrays.update({f"setup__{k}": setup[k] for k in ("switches", "fluid")})
            for key, f in (("cells_vtk", "solution.vtk"), ("bc_vtk", "solution_BC.vtk")):
                with open(os.path.join(d, f), "rb") as fh:
                    arrays[key] = np.frombuffer(fh.read(), np.uint8)
        mesh_args = spec["mesh"]
        arrays["mesh_dims"] = np.array([mesh_args[k] for k in ("nx", "ny", "nz")])
        arrays["mesh_lengths"] = np.array(mesh_args["lengths"], float)
        arrays["mesh_jitter"] = np.array(float(mesh_args["jitter"]))
        arrays["mesh_cells"] = np.array(spec["cells"])
        np.savez_compressed(os.path.join(out_dir, f"vtk_{name}.npz"), **arrays)
    # heat conduction on a hex box (oracle/ref_assembly.cpp, case heat3d): the
    # reference's own run_config writes the VTK files into its working directory
    exe = os.path.join(ROOT, "oracle", "_ref", "ref_assembly")
    mesh = {"nx": 6, "ny": 5, "nz": 4, "lengths": (1.0, 0.2, 0.1), "jitter": 0.1}
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "m.su2")
        m = dict(mesh)
        W.write_su2_box(path, m.pop("nx"), m.pop("ny"), m.pop("nz"), cells="hex", **m)
        subprocess.run([exe, d, f"heat3d={path}", "0", "0"], cwd=d, check=True,
                       stdout=subprocess.DEVNULL)
        arrays = {f"final__{k}": v
                  for k, v in read_named_arrays(os.path.join(d, "final_heat.bin")).items()}
        for key, f in (("cells_vtk", "solution.vtk"), ("bc_vtk", "solution_BC.vtk")):
            with open(os.path.join(d, f), "rb") as fh:
                arrays[key] = np.frombuffer(fh.read(), np.uint8)
    arrays["mesh_dims"] = np.array([mesh[k] for k in ("nx", "ny", "nz")])
    arrays["mesh_lengths"] = np.array(mesh["lengths"], float)
    arrays["mesh_jitter"] = np.array(float(mesh["jitter"]))
    arrays["mesh_cells"] = np.array("hex")
    np.savez_compressed(os.path.join(out_dir, "vtk_heat.npz"), **arrays)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=orc.REF_DIR)
    ap.add_argument("--only", choices=["kat", "shocktube", "small", "assembly", "flow", "mesh",
                                       "vtk"],
                    help="write one fixture (default: all)")
    a = ap.parse_args()
    orc.build(a.reference)
    ref = orc.Reference()
    ref.set_threads(1)
    want = lambda name: a.only in (None, name)  # noqa: E731
    if want("kat"):
        make_kat(ref, os.path.join(HERE, "kat_tridiag10.npz"))
    if want("shocktube"):
        make_shocktube(os.path.join(HERE, "shocktube_calls.npz"))
    if want("small"):
        make_small(ref, os.path.join(HERE, "small_systems.npz"))
    if want("assembly"):
        make_assembly(HERE)
    if want("flow"):
        for case in FLOW_CASES:
            make_flow(HERE, case)
    if want("mesh"):
        make_meshes(HERE)
    if want("vtk"):
        make_vtk(HERE)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
