"""VTK output (ocsl_vtk_write, Mesh.write_vtk) against the reference's own
files: solution.vtk and solution_BC.vtk as Cpost_processing writes them
(cpost_processing.cpp:26-401), recorded by oracle/ref_flow.cpp after short
runs of the 3D viscous channel on jittered boxes of hexahedra, tetrahedra and
wedges read from SU2 files (tests/golden/vtk_<cells>.npz, made by
tests/golden/make_golden.py).

* CPU: from the recorded final state in host memory, both files are
  byte-identical to the reference's, for every cell kind and for a heat-
  conduction run (oracle/ref_assembly.cpp, case heat3d); 17 digits give the
  state back bit for bit; the heat-conduction branch writes the reference's
  sections; missing fields, bad digit counts and unwritable paths are refused.
* GPU: the same state as CUDA tensors (streamed from the device) gives the
  same bytes; and the device SIMPLE loop's own state after the recorded 3D
  run, written from device memory, matches the reference's files number by
  number within the run's agreement with the reference (1e-11 of each field's
  scale) plus the 6-digit print rounding.
"""
import os

import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("hex", "tet", "wedge")


def fixture(name):
    return np.load(os.path.join(GOLDEN, f"vtk_{name}.npz"))


def write_mesh(z, path):
    nx, ny, nz = (int(v) for v in z["mesh_dims"])
    W.write_su2_box(path, nx, ny, nz, cells=str(z["mesh_cells"]),
                    lengths=tuple(float(v) for v in z["mesh_lengths"]),
                    jitter=float(z["mesh_jitter"]))


def flow_fields(z, to=lambda a: a):
    fl, sw = z["setup__fluid"], z["setup__switches"]
    return dict(density=to(z["final__cell_density"]), pressure=to(z["final__cell_pressure"]),
                temperature=to(z["final__cell_temperature"]), mach=to(z["final__cell_mach"]),
                velocity=to(z["final__cell_velocity"]),
                pressure_grad=to(z["final__cell_pressure_grad"]),
                bc_type=to(z["final__bc_type"]), bc_wall=to(z["final__bc_wall"]),
                viscous=bool(sw[0]), sutherland=(float(fl[2]), float(fl[3])))


def sections(text: str) -> dict:
    """Keyword line -> rows of numbers that follow it (a SCALARS section's
    LOOKUP_TABLE line belongs to its header)."""
    out, key = {}, None
    for line in text.splitlines():
        if line.startswith("LOOKUP_TABLE"):
            continue
        if line[:1].isalpha() or line.startswith("#"):
            key = line
            assert key not in out, key
            out[key] = []
        elif key is not None:
            out[key].append([float(v) for v in line.split()])
    return out


@pytest.mark.parametrize("name", CASES)
def test_vtk_bytes_equal_reference(lib_built, tmp_path, name):
    z = fixture(name)
    write_mesh(z, tmp_path / "m.su2")
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        m.write_vtk(tmp_path / "c.vtk", tmp_path / "b.vtk", **flow_fields(z))
    assert (tmp_path / "c.vtk").read_bytes() == bytes(z["cells_vtk"])
    assert (tmp_path / "b.vtk").read_bytes() == bytes(z["bc_vtk"])


def heat_fields(z, to=lambda a: a):
    return dict(heat=True, temperature=to(z["final__cell_temperature"]),
                bc_temperature=to(z["final__bc_temperature"]))


def test_vtk_heat_bytes_equal_reference(lib_built, tmp_path):
    """A heat-conduction run of the reference on a hex box (inlet 250 K, outlet
    450 K, adiabatic walls): its solution.vtk / solution_BC.vtk."""
    z = fixture("heat")
    write_mesh(z, tmp_path / "m.su2")
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        m.write_vtk(tmp_path / "c.vtk", tmp_path / "b.vtk", **heat_fields(z))
    assert (tmp_path / "c.vtk").read_bytes() == bytes(z["cells_vtk"])
    assert (tmp_path / "b.vtk").read_bytes() == bytes(z["bc_vtk"])


def test_vtk_full_precision_round_trips(lib_built, tmp_path):
    z = fixture("hex")
    write_mesh(z, tmp_path / "m.su2")
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        m.write_vtk(tmp_path / "c.vtk", tmp_path / "b.vtk", digits=17, **flow_fields(z))
    s = sections((tmp_path / "c.vtk").read_text())
    n = z["final__cell_density"].size
    got = np.array(s["SCALARS Density[Kg/m^3] double 1"]).ravel()
    assert np.array_equal(got, z["final__cell_density"])
    vel = np.array(s["VECTORS Velocity[m/s] double"]).T.ravel()
    assert np.array_equal(vel, z["final__cell_velocity"].reshape(3, n).ravel())
    # the reference's 6-digit file says the same to its precision
    ref = sections(bytes(z["cells_vtk"]).decode())
    np.testing.assert_allclose(np.array(ref["VECTORS Velocity[m/s] double"]).T.ravel(), vel,
                               rtol=5e-6, atol=0)


def test_vtk_heat_sections(lib_built, tmp_path):
    z = fixture("tet")
    write_mesh(z, tmp_path / "m.su2")
    T = z["final__cell_temperature"]
    Tb = z["final__bc_temperature"]
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        m.write_vtk(tmp_path / "c.vtk", tmp_path / "b.vtk", heat=True, digits=17,
                    temperature=T, bc_temperature=Tb)
    c = sections((tmp_path / "c.vtk").read_text())
    b = sections((tmp_path / "b.vtk").read_text())
    # cpost_processing.cpp:41-48 and :162-169: Temperature after the geometry
    assert list(c)[-2:] == ["VECTORS Center double", "SCALARS Temperature[K] double 1"]
    assert list(b)[-2:] == ["Vectors center double", "SCALARS Temperature[K] double 1"]
    assert np.array_equal(np.array(c["SCALARS Temperature[K] double 1"]).ravel(), T)
    assert np.array_equal(np.array(b["SCALARS Temperature[K] double 1"]).ravel(), Tb)
    # at 6 digits everything before the temperature is the flow file's geometry
    ref = bytes(z["cells_vtk"]).decode()
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        m.write_vtk(tmp_path / "c6.vtk", None, heat=True, temperature=T)
    assert (tmp_path / "c6.vtk").read_text().split("SCALARS Temperature")[0] == \
        ref.split("SCALARS Density")[0]


def test_vtk_refuses_bad_input(lib_built, tmp_path):
    z = fixture("wedge")
    write_mesh(z, tmp_path / "m.su2")
    f = flow_fields(z)
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        with pytest.raises(ocsl.OcslError, match="missing"):
            m.write_vtk(tmp_path / "c.vtk", None, **dict(f, mach=None))
        with pytest.raises(ocsl.OcslError, match="missing"):
            m.write_vtk(None, tmp_path / "b.vtk", **dict(f, bc_wall=None))
        with pytest.raises(ocsl.OcslError, match="digits"):
            m.write_vtk(tmp_path / "c.vtk", None, digits=18, **f)
        with pytest.raises(ocsl.OcslError, match="cannot open"):
            m.write_vtk(tmp_path / "no_such_dir" / "c.vtk", None, **f)
        with pytest.raises(ocsl.OcslError, match="bc_temperature"):
            m.write_vtk(None, tmp_path / "b.vtk", heat=True, temperature=f["temperature"])
        # nothing requested: nothing written, no error
        m.write_vtk(None, None, **f)


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES + ("heat",))
def test_vtk_from_device_equals_reference(lib_built, torch_cuda, tmp_path, name):
    torch = torch_cuda
    z = fixture(name)
    write_mesh(z, tmp_path / "m.su2")

    def dev(a):
        return torch.from_numpy(np.ascontiguousarray(a)).cuda()

    fields = heat_fields(z, dev) if name == "heat" else flow_fields(z, dev)
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        m.write_vtk(tmp_path / "c.vtk", tmp_path / "b.vtk", **fields)
    assert (tmp_path / "c.vtk").read_bytes() == bytes(z["cells_vtk"])
    assert (tmp_path / "b.vtk").read_bytes() == bytes(z["bc_vtk"])


@pytest.mark.gpu
def test_vtk_of_device_simple_run_matches_reference(ctx, torch_cuda, tmp_path):
    """The 3D viscous channel run on the device with the reference's solvers
    (40 steps x 3 inner iterations), its state written from device memory."""
    import flow_cases as FC

    z = fixture("hex")
    g = FC.Golden("box3d")
    assert (g.steps, g.inner) == (40, 3)
    dev = FC.DeviceCase(torch_cuda, g.case())
    dev.bind(ctx)
    methods = (ocsl.BICGSTAB_REF, ocsl.BICGSTAB_REF, ocsl.BICGSTAB_REF)
    for _ in range(g.steps):
        for _ in range(g.inner):
            assert dev.iterate(ctx, methods)["status"] == [0] * 5
        dev.end_step(ctx)
    torch_cuda.cuda.synchronize()
    write_mesh(z, tmp_path / "m.su2")
    st, ar = dev.state, dev.arrays
    fl, sw = z["setup__fluid"], z["setup__switches"]
    with ocsl.Mesh(str(tmp_path / "m.su2")) as m:
        m.write_vtk(tmp_path / "c.vtk", tmp_path / "b.vtk", density=st["density_c"],
                    pressure=st["pressure"], temperature=st["temperature"], mach=ar["mach"],
                    velocity=st["velocity"], pressure_grad=st["pressure_grad"],
                    bc_type=st["bc_type"], bc_wall=st["bc_wall"], viscous=bool(sw[0]),
                    sutherland=(float(fl[2]), float(fl[3])))
    for mine, ref in (("c.vtk", "cells_vtk"), ("b.vtk", "bc_vtk")):
        a = sections((tmp_path / mine).read_text())
        b = sections(bytes(z[ref]).decode())
        assert list(a) == list(b)
        for key in b:
            x, y = np.array(a[key], float), np.array(b[key], float)
            assert x.shape == y.shape, key
            if not y.size:
                continue
            scale = float(np.max(np.abs(y)))
            tol = 1e-11 * scale + 1e-5 * np.abs(y)  # two 6-digit roundings
            assert np.all(np.abs(x - y) <= tol), (mine, key, float(np.max(np.abs(x - y))))
