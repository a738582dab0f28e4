"""The SIMPLE inner iteration on the device (ocsl_flow_iterate_device) on the
reference's recorded runs (tests/golden/flow_<case>.npz): the 1000-cell
inviscid shock tube, the 200-cell viscous channel (velocity inlet, no-slip
walls, pressure outlet) and steady (supersonic inlet, slip walls, outlet,
implicit under-relaxation ramp) cases, and a 3D viscous channel on a
240-cell jittered hex mesh read by the reference from an SU2 file.

* Bit-exact to the oracle restatement, inner iteration by inner iteration
  (every field the iteration writes, the residual sums and the solves'
  iteration counts), with the reference's own solvers (momentum CG_solve or
  ILU_BICGSTAB_solve; p' and enthalpy ILU_BICGSTAB_solve) and with the
  tolerance-mode ILU-BiCGSTAB.
* Whole recorded runs against the reference's final fields, with the
  reference's solvers: the state (p, u, T, rho, h, mass fluxes) within 1e-11
  relative (measured: a few 1e-13 on the shock tube, the residue of the
  reference's -ffast-math build and its serial dot products), every field
  within 1e-8 (pressure gradients, p' and cell mass balances are differences
  of nearly equal pressures).  With every equation solved by the
  tolerance-mode ILU-BiCGSTAB to 1e-10, or by the FP32-inner / FP64-refined
  one, the state within 5e-9 of the reference run that uses
  ILU_BICGSTAB_solve everywhere (measured 1.1e-9 on the shock tube: the
  reference's own solves stop after a fixed count; p' and its gradient,
  nearly zero in a settled flow, are reported, not bounded); with those
  solves run through the multicolour ordering (another ILU(0) factor, the
  same residual), within 1e-7 (measured 2.3e-8 on the shock tube).
* Input the iteration cannot take is refused before anything is written.
"""
import time

import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from oracle import oracle as orc

import flow_cases as FC

pytestmark = pytest.mark.gpu

METHODS = {
    "bicg": (ocsl.BICGSTAB_REF, ocsl.BICGSTAB_REF, ocsl.BICGSTAB_REF),
    "cg": (ocsl.CG_REF, ocsl.BICGSTAB_REF, ocsl.BICGSTAB_REF),
    "tol": (ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB),
    "ir32": (ocsl.ILU_BICGSTAB_IR32, ocsl.ILU_BICGSTAB_IR32, ocsl.ILU_BICGSTAB_IR32),
}
# the tolerance modes again through the multicolour ordering (ocsl_set_ordering)
METHODS["tol_mc"] = METHODS["tol"]
METHODS["ir32_mc"] = METHODS["ir32"]
STATE = ("velocity", "pressure", "temperature", "density_c", "enthalpy", "mdot", "density",
         "bc_mdot", "bc_density", "bc_enthalpy", "bc_temperature", "bc_velocity", "bc_pressure")

_golden = {}


def golden(case="shocktube"):
    if case not in _golden:
        _golden[case] = FC.Golden(case)
    return _golden[case]


def _oracle_end_step(c):
    FC.end_step(c, orc.flow_end_step)


def _same(got: dict, want: dict, where):
    for k in want:
        assert np.array_equal(got[k], want[k]), (where, k, FC.relerr(got[k], want[k]))


@pytest.mark.parametrize("case,mode", [("shocktube", "bicg"), ("shocktube", "cg"),
                                       ("shocktube", "tol"), ("channel", "bicg"),
                                       ("channel", "tol"), ("steady", "bicg"), ("steady", "tol"),
                                       ("box3d", "bicg"), ("box3d", "cg"), ("box3d", "tol")])
def test_iteration_bit_exact_vs_oracle(ctx, torch_cuda, case, mode):
    g = golden(case)
    c = g.case()
    dev = FC.DeviceCase(torch_cuda, g.case())
    dev.bind(ctx)
    for step in range(2 if g.inner > 1 else 4):
        for inner in range(g.inner):
            rep = dev.iterate(ctx, METHODS[mode])
            want = orc.flow_iterate(c, METHODS[mode])
            _same(dev.written(), FC.written(c), (case, mode, step, inner))
            assert rep["residual"] == list(want["residual"]), (case, mode, step, inner, rep)
            assert rep["iterations"] == list(want["iterations"]), (case, mode, step, inner, rep)
            assert rep["status"] == [0] * 5
        dev.end_step(ctx)
        _oracle_end_step(c)
        assert dev.case["eq"] == c["eq"]
    for k in ("velocity_last", "density_last", "pressure_last", "enthalpy_last"):
        assert np.array_equal(dev.state[k].cpu().numpy(), c["state"][k]), k


@pytest.mark.parametrize("case,mode", [("shocktube", "bicg"), ("shocktube", "cg"),
                                       ("shocktube", "tol"), ("shocktube", "ir32"),
                                       ("channel", "bicg"), ("channel", "tol"),
                                       ("steady", "bicg"), ("steady", "ir32"),
                                       ("box3d", "bicg"), ("box3d", "tol"),
                                       ("shocktube", "tol_mc"), ("channel", "ir32_mc"),
                                       ("steady", "tol_mc"), ("box3d", "ir32_mc")])
def test_recorded_run_vs_reference(ctx, torch_cuda, case, mode):
    g = golden(case)
    dev = FC.DeviceCase(torch_cuda, g.case())
    dev.bind(ctx)
    if mode.endswith("_mc"):
        ctx.set_ordering("multicolour")
    torch_cuda.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(g.steps):
        for _ in range(g.inner):
            rep = dev.iterate(ctx, METHODS[mode])
            assert rep["status"] == [0] * 5, rep
        dev.end_step(ctx)
    torch_cuda.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / (g.steps * g.inner)
    ref = "final_cg" if mode == "cg" else "final_bicg"
    errs = FC.field_errors(dev.written(), FC.recorded(g.setup, g.record(ref)))
    state = max(errs[k] for k in STATE)
    print(f"{case} {mode}: {ms:.3f} ms per inner iteration; vs {ref}: state {state:.2e}, "
          f"all fields {max(errs.values()):.2e} ({max(errs, key=errs.get)})")
    if mode in ("bicg", "cg"):
        assert state <= 1e-11, errs
        assert max(errs.values()) <= 1e-8, errs
    else:
        # converged solves against fixed-count ones: the state; the derived
        # fields of a nearly settled p' carry no meaningful relative error.
        # Through the multicolour ordering the solves reach the same 1e-10
        # residual with another factor, so their solutions differ from the
        # natural-order ones within the conditioning of each equation
        # (measured 2.3e-8 in the shock tube's enthalpy over 1000 iterations)
        assert state <= (1e-7 if mode.endswith("_mc") else 5e-9), errs


def test_rejects_unsupported_input(ctx, torch_cuda):
    g = golden()
    dev = FC.DeviceCase(torch_cuda, g.case())
    dev.bind(ctx)
    before = {k: v.clone() for k, v in dev.state.items()}
    kinds = dev.state["bc_type"].clone()
    kinds[3] = 9  # not an ocsl_bc_type
    dev.state["bc_type"] = kinds
    with pytest.raises(ocsl.OcslError) as e:
        dev.iterate(ctx, METHODS["bicg"])
    assert e.value.status == _abi.BAD_ARGUMENT
    dev.state["bc_type"] = before["bc_type"]
    state = dict(dev.state)
    del state["stress"]  # a viscous flow needs the stress array
    with pytest.raises(ocsl.OcslError) as e:
        ctx.flow_iterate_device(dict(dev.case["eq"], viscous=1), state, dev.arrays,
                                dev.case["constants"], METHODS["bicg"])
    assert e.value.status == _abi.BAD_ARGUMENT
    arrays = dict(dev.arrays)
    del arrays["bc_alpha"]
    with pytest.raises(ocsl.OcslError) as e:
        ctx.flow_iterate_device(dev.case["eq"], dev.state, arrays, dev.case["constants"],
                                METHODS["bicg"])
    assert e.value.status == _abi.BAD_ARGUMENT
    for k, v in before.items():
        assert torch_cuda.equal(dev.state[k], v), k
    # the context still iterates exactly like the oracle
    c = g.case()
    dev.iterate(ctx, METHODS["bicg"])
    orc.flow_iterate(c, METHODS["bicg"])
    _same(dev.written(), FC.written(c), "after refusals")


def test_graph_replay_matches_direct_launches(ctx, torch_cuda):
    """Reference-faithful iterations run as one captured CUDA graph from the
    second call with the same arguments on; the graph (this context), the
    direct launches (a context with graphs off) and the oracle agree bit for
    bit, on torch's default stream and on a side stream (a new key each
    switch), and a changed constant is captured afresh."""
    torch = torch_cuda
    g = golden()
    case = g.case()
    graphed, direct = FC.DeviceCase(torch, g.case()), FC.DeviceCase(torch, g.case())
    graphed.bind(ctx)
    ctx2 = ocsl.Context(0)
    try:
        ctx2.set_graphs(False)
        direct.bind(ctx2)
        side = torch.cuda.Stream()
        for k in range(12):
            if k == 8:  # a new under-relaxation factor: a new key
                for c in (case, graphed.case, direct.case):
                    c["constants"] = dict(c["constants"], relax_u=0.9)
            if 4 <= k < 8:
                with torch.cuda.stream(side):
                    r0 = graphed.iterate(ctx, METHODS["cg"])
                side.synchronize()
            else:
                r0 = graphed.iterate(ctx, METHODS["cg"])
            r1 = direct.iterate(ctx2, METHODS["cg"])
            want = orc.flow_iterate(case, METHODS["cg"])
            _same(graphed.written(), FC.written(case), ("graph", k))
            _same(direct.written(), FC.written(case), ("direct", k))
            assert r0 == r1, (k, r0, r1)
            assert r0["residual"] == list(want["residual"])
            assert r0["iterations"] == list(want["iterations"])
    finally:
        ctx2.close()


def test_su2_mesh_to_device_iteration(ctx, torch_cuda, tmp_path):
    """The whole chain from the mesh file: the SU2 file the reference read,
    turned into finite-volume arrays and the matrix pattern by the library's
    own reader, drives the recorded 3D run on the device; the final state
    meets the reference's within 1e-11 (the reader's metrics differ from the
    reference's -ffast-math ones by ~1e-14)."""
    from opencslsolver_gb300 import workloads as W

    g = golden("box3d")
    path = str(tmp_path / "box3d.su2")
    W.write_su2_box(path, 10, 6, 4)
    m = ocsl.read_su2(path)
    rp, col = ocsl.build_pattern(m["n_cells"], m["face_left"], m["face_right"], m["bc_left"])
    setup = dict(g.setup, row_ptr=rp, column_index=col)
    for k in ("face_left", "face_right", "bc_left", "face_geo_aver", "face_ksi_A",
              "face_area_vector", "face_alpha", "face_distance", "face_unit", "bc_area",
              "bc_area_vector", "bc_alpha", "bc_distance", "bc_unit", "bc_perp_dist", "bc_ksi_A"):
        setup[k] = m[k]
    setup["cell_volume"] = m["cell_volume"]
    dev = FC.DeviceCase(torch_cuda, FC.make_case(setup, g.setup))
    dev.bind(ctx)
    for _ in range(g.steps):
        for _ in range(g.inner):
            assert dev.iterate(ctx, METHODS["bicg"])["status"] == [0] * 5
        dev.end_step(ctx)
    errs = FC.field_errors(dev.written(), FC.recorded(g.setup, g.record("final_bicg")))
    assert max(errs[k] for k in STATE) <= 1e-11, errs
    assert max(errs.values()) <= 1e-8, errs


@pytest.mark.parametrize("cells", ["hex", "tet", "wedge"])
def test_flow_run_from_su2_bit_exact_vs_oracle(ctx, torch_cuda, tmp_path, cells):
    """The user path without the reference: SU2 file -> read_su2 ->
    build_pattern -> flow.initial_state -> FlowRun on the device, for
    hexahedra (structured sweeps), tetrahedra (level-scheduled sweeps) and
    wedges; every inner iteration and time step equals the oracle's on the
    same case bit for bit, with the reference's and the tolerance-mode
    solvers."""
    import copy

    from opencslsolver_gb300 import flow as F
    from opencslsolver_gb300 import workloads as W

    path = str(tmp_path / "m.su2")
    W.write_su2_box(path, 6, 5, 4, cells=cells)
    mesh = ocsl.read_su2(path)
    rp, col = ocsl.build_pattern(mesh["n_cells"], mesh["face_left"], mesh["face_right"],
                                 mesh["bc_left"])
    mesh.update(row_ptr=rp, column_index=col)
    case = F.initial_state(mesh, **FC.CONFIGS["box3d"])
    for mode in ("bicg", "tol"):
        c = copy.deepcopy(case)
        run = F.FlowRun(ctx, copy.deepcopy(case))
        for step in range(2):
            for inner in range(3):
                rep = run.iterate(METHODS[mode])
                want = orc.flow_iterate(c, METHODS[mode])
                got = {k: run.state[k].cpu().numpy() for k in FC.WRITTEN_STATE}
                got.update({k: run.arrays[k].cpu().numpy() for k in FC.WRITTEN_ARRAYS})
                _same(got, FC.written(c), (cells, mode, step, inner))
                assert rep["residual"] == list(want["residual"]), (cells, mode, rep)
                assert rep["iterations"] == list(want["iterations"]), (cells, mode, rep)
            run.end_step()
            FC.end_step(c, orc.flow_end_step)


@pytest.mark.parametrize("case", ["shocktube", "box3d"])
def test_ir32_iteration_graph_equals_direct(ctx, torch_cuda, case):
    """With ocsl_set_device_loop the SIMPLE iteration with FP32-refined solves
    is one CUDA graph too (from the second call; the solves' loops as
    conditional graph nodes): every field, residual, iteration count and
    status equals the directly launched iteration's, step by step; the time
    per inner iteration of both is printed."""
    torch = torch_cuda
    g = golden(case)
    steps = 3
    runs = {}
    for dev_loop in (False, True):
        dev = FC.DeviceCase(torch, g.case())
        dev.bind(ctx)
        ctx.set_device_loop(dev_loop)
        stream = torch.cuda.Stream()
        reps, fields = [], []
        with torch.cuda.stream(stream):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(steps):
                for _ in range(g.inner):
                    reps.append(dev.iterate(ctx, METHODS["ir32"]))
                    fields.append(dev.written())
                dev.end_step(ctx)
            stream.synchronize()
            ms = (time.perf_counter() - t0) * 1e3 / (steps * g.inner)
        runs[dev_loop] = (reps, fields, ms)
    ctx.set_device_loop(False)
    (r0, f0, ms0), (r1, f1, ms1) = runs[False], runs[True]
    for k, (a, b) in enumerate(zip(r0, r1)):
        assert a["status"] == b["status"] == [0] * 5, (k, a, b)
        assert a["iterations"] == b["iterations"] and a["residual"] == b["residual"], (k, a, b)
    for k, (a, b) in enumerate(zip(f0, f1)):
        _same(b, a, (case, k))
    print(f"{case}: FP32-refined SIMPLE iteration {ms0:.2f} ms direct, {ms1:.2f} ms as one graph "
          f"(host wall clock, first calls included)")
