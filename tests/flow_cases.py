"""Flow cases for the SIMPLE-iteration tests: the reference's recorded states
of the shock tube, the viscous channel and steady cases and a 3D viscous
channel on an SU2 hex mesh
(tests/golden/flow_<case>.npz, written by tests/golden/make_golden.py from
oracle/ref_flow.cpp's dumps) turned into the library's ocsl_flow_state /
ocsl_flow_iteration layout, and the reference's own driver logic around the
iteration (update_timestep and its under-relaxation ramp)."""
import os

import numpy as np

from opencslsolver_gb300 import _abi

# ocsl_flow_state field <- recorded name
STATE_FROM = {
    "geo_aver": "face_geo_aver", "ksi_A": "face_ksi_A", "mdot": "face_mdot",
    "density": "face_density", "qy": "face_qy", "stress": "face_stress",
    "bc_type": "bc_type", "bc_wall": "bc_wall", "bc_supersonic": "bc_supersonic",
    "bc_area": "bc_area", "bc_area_vector": "bc_area_vector", "bc_perp_dist": "bc_perp_dist",
    "bc_ksi_A": "bc_ksi_A", "bc_mdot": "bc_mdot", "bc_density": "bc_density", "bc_qy": "bc_qy",
    "bc_temperature": "bc_temperature", "bc_enthalpy": "bc_enthalpy",
    "bc_velocity": "bc_velocity", "volume": "cell_volume", "delta_t": "cell_delta_t",
    "velocity": "cell_velocity", "velocity_last": "cell_velocity_last",
    "pressure_grad": "cell_pressure_grad", "density_c": "cell_density",
    "density_last": "cell_density_last", "pressure": "cell_pressure",
    "pressure_last": "cell_pressure_last", "pressure_corr": "cell_pressure_corr",
    "temperature": "cell_temperature", "enthalpy": "cell_enthalpy",
    "enthalpy_last": "cell_enthalpy_last", "bc_thermal": "bc_thermal",
}
# ocsl_flow_iteration array <- recorded name
ARRAYS_FROM = {
    "face_area_vector": "face_area_vector", "face_alpha": "face_alpha",
    "face_distance": "face_distance", "face_unit": "face_unit", "bc_distance": "bc_distance",
    "bc_unit": "bc_unit", "bc_alpha": "bc_alpha", "bc_out_pressure": "bc_out_pressure",
    "bc_pressure": "bc_pressure",
    "pressure_corr_grad": "cell_pressure_corr_grad", "ap": "cell_ap", "ap_vec": "cell_ap_vec",
    "mach": "cell_mach", "total_mdot": "cell_total_mdot",
}
# geometry: taken from the setup record, never changed by the iteration
SETUP_ONLY = {"geo_aver", "ksi_A", "bc_area", "bc_area_vector", "bc_perp_dist", "bc_ksi_A",
              "volume", "face_area_vector", "face_alpha", "face_distance", "face_unit",
              "bc_distance", "bc_unit", "bc_alpha"}
GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("shocktube", "channel", "steady", "box3d")
# recorded inner iterations (step_iteration) of each fixture
ITERATIONS = {"shocktube": ("0_0", "0_1", "57_2"), "channel": ("0_0", "0_1", "40_1"),
              "steady": ("0_0", "1_0", "10_0"), "box3d": ("0_0", "0_1", "20_1")}

# the fields one inner iteration writes (compared after it)
WRITTEN_STATE = ("velocity", "density_c", "pressure", "pressure_grad", "pressure_corr",
                 "temperature", "enthalpy", "mdot", "density", "qy", "stress", "bc_mdot",
                 "bc_density", "bc_qy", "bc_enthalpy", "bc_supersonic", "bc_temperature",
                 "bc_velocity")
WRITTEN_ARRAYS = ("bc_pressure", "pressure_corr_grad", "ap", "ap_vec", "mach", "total_mdot")


def make_case(setup: dict, rec: dict) -> dict:
    """A flow case: the mesh, switches and constants of ``setup`` with the
    state of ``rec`` (a state record), every array a fresh contiguous copy."""
    fl = setup["fluid"]
    visc, blended, transient = (int(v) for v in setup["switches"])
    relax = float(rec["implicit_underrelaxation"][0])
    state, arrays = {}, {}
    for k, name in STATE_FROM.items():
        src = setup if k in SETUP_ONLY else rec
        dt = np.int32 if k in _abi.INT_FIELDS else np.float64
        state[k] = np.ascontiguousarray(src[name], dt).copy()
    for k, name in ARRAYS_FROM.items():
        src = setup if k in SETUP_ONLY else rec
        arrays[k] = np.ascontiguousarray(src[name], np.float64).copy()
    return {
        "row_ptr": setup["row_ptr"], "column_index": setup["column_index"],
        "left": setup["face_left"], "right": setup["face_right"], "bc_left": setup["bc_left"],
        "eq": {"viscous": visc, "blended": blended, "transient": transient,
               "R_specific": fl[0], "gamma": fl[1], "sutherland": (fl[2], fl[3]),
               "prandtl": fl[4], "implicit_underrelaxation": relax},
        "ramp": tuple(float(v) for v in setup["relax_ramp"]),
        "constants": {"cp": fl[6], "Tref": fl[7], "H_formation": fl[8], "relax_p": fl[9],
                      "relax_u": fl[10]},
        "state": state, "arrays": arrays,
    }


def written(case: dict) -> dict:
    """The fields one inner iteration writes, by name."""
    out = {k: case["state"][k] for k in WRITTEN_STATE}
    out.update({k: case["arrays"][k] for k in WRITTEN_ARRAYS})
    return out


def recorded(setup: dict, rec: dict) -> dict:
    """The same fields from a state record."""
    c = make_case(setup, rec)
    return written(c)


def end_step(case: dict, end_step_fn) -> None:
    """The rest of CFlow_solver::update_timestep (cflow_solver.cpp:503-519)
    after ``end_step_fn`` copied the fields to their *_last: the steady
    under-relaxation ramp, with the reference's own arithmetic."""
    end_step_fn(case)
    eq = case["eq"]
    init, top, steps = case["ramp"]
    if not eq["transient"] and eq["implicit_underrelaxation"] < top:
        eq["implicit_underrelaxation"] += (top - init) / steps


class Golden:
    """tests/golden/flow_<case>.npz, by record."""

    def __init__(self, case: str = "shocktube"):
        z = np.load(os.path.join(GOLDEN_DIR, f"flow_{case}.npz"))
        self.name = case
        self._z = {k: z[k] for k in z.files}
        self.steps, self.inner = (int(v) for v in self._z["run"])
        self.iterations = ITERATIONS[case]

    def record(self, prefix: str) -> dict:
        p = prefix + "__"
        return {k[len(p):]: v for k, v in self._z.items() if k.startswith(p)}

    @property
    def setup(self) -> dict:
        return self.record("setup")

    def start(self, tag: str) -> dict:
        return self.setup if tag == "0_0" else self.record(f"start_{tag}")

    def start_case(self, tag: str, end_step_fn) -> dict:
        """The case right before inner iteration ``tag``, with the
        under-relaxation the reference used in it."""
        c = self.case(self.start(tag))
        if tag != "0_0" and int(self._z[f"endstep_{tag}"]):
            end_step_fn(c)
        c["eq"]["implicit_underrelaxation"] = float(self._z[f"relax_{tag}"][0])
        return c

    def systems(self, tag: str) -> dict:
        return {k: self._z[f"{k}_{tag}"] for k in ("value", "b", "x0", "x")}

    def case(self, record: dict | None = None) -> dict:
        return make_case(self.setup, self.setup if record is None else record)


def relerr(got, want) -> float:
    scale = float(np.max(np.abs(want))) if np.size(want) else 0.0
    return float(np.max(np.abs(np.asarray(got) - np.asarray(want)))) / (scale or 1.0)


def field_errors(got: dict, want: dict) -> dict:
    """Max |got - want| / max |want| per field (the supersonic flags exactly)."""
    return {k: (float(not np.array_equal(got[k], want[k])) if k == "bc_supersonic"
                else relerr(got[k], want[k])) for k in want}


class DeviceCase:
    """A flow case's arrays as CUDA tensors, for Context.flow_iterate_device."""

    def __init__(self, torch, case: dict):
        self.torch = torch
        self.case = case

        def dev(k, v):
            dt = torch.int32 if k in _abi.INT_FIELDS else torch.float64
            return torch.from_numpy(np.ascontiguousarray(v)).to(device="cuda", dtype=dt)

        self.state = {k: dev(k, v) for k, v in case["state"].items()}
        self.arrays = {k: dev(k, v) for k, v in case["arrays"].items()}

    def bind(self, ctx) -> None:
        c = self.case
        ctx.set_pattern(c["row_ptr"], c["column_index"])
        ctx.set_faces(c["left"], c["right"], c["bc_left"])

    def iterate(self, ctx, methods, **opts) -> dict:
        return ctx.flow_iterate_device(self.case["eq"], self.state, self.arrays,
                                       self.case["constants"], methods, **opts)

    def end_step(self, ctx) -> None:
        end_step(self.case, lambda c: ctx.flow_end_step_device(self.state))

    def written(self) -> dict:
        out = {k: self.state[k].cpu().numpy() for k in WRITTEN_STATE}
        out.update({k: self.arrays[k].cpu().numpy() for k in WRITTEN_ARRAYS})
        return out


# The configurations oracle/ref_flow.cpp runs (shocktube_config.h, flow_configs.h),
# as opencslsolver_gb300.flow.initial_state arguments.
CONFIGS = {
    "shocktube": dict(initial={"pressure": 1e5, "temperature": 348.4, "velocity": (0, 0, 0),
                               "pressure2": 1e4, "temperature2": 278.7},
                      boundaries=[{"kind": "wall", "wall": "slip"}, {"kind": "empty"},
                                  {"kind": "wall", "wall": "slip"}],
                      viscous=False, blended=True, transient=True, dt=1e-6),
    "channel": dict(initial={"pressure": 1e5, "temperature": 300.0, "velocity": (20, 0, 0)},
                    boundaries=[{"kind": "velocity_inlet", "velocity": (20, 0, 0),
                                 "temperature": 300.0, "pressure": 1e5},
                                {"kind": "wall", "wall": "no_slip"},
                                {"kind": "pressure_outlet", "pressure": 1e5}],
                    viscous=True, blended=False, transient=True, dt=1e-5),
    "steady": dict(initial={"pressure": 1e5, "temperature": 300.0, "velocity": (700, 0, 0)},
                   boundaries=[{"kind": "supersonic_inlet", "velocity": (700, 0, 0),
                                "temperature": 300.0, "pressure": 1e5},
                               {"kind": "wall", "wall": "slip"},
                               {"kind": "pressure_outlet", "pressure": 1e5}],
                   viscous=True, blended=True, transient=False, dt=1e-5),
    "box3d": dict(initial={"pressure": 1e5, "temperature": 300.0, "velocity": (20, 0, 0)},
                  boundaries=[{"kind": "velocity_inlet", "velocity": (20, 3, 2),
                               "temperature": 300.0, "pressure": 1e5},
                              {"kind": "wall", "wall": "no_slip"},
                              {"kind": "pressure_outlet", "pressure": 1e5}],
                  viscous=True, blended=True, transient=True, dt=2e-6),
}


def mesh_from_setup(setup: dict) -> dict:
    """The recorded finite-volume arrays in the form of read_su2's output."""
    keys = ("face_left", "face_right", "face_geo_aver", "face_ksi_A", "face_area_vector",
            "face_alpha", "face_distance", "face_unit", "bc_left", "bc_marker", "bc_area",
            "bc_area_vector", "bc_alpha", "bc_distance", "bc_unit", "bc_perp_dist", "bc_ksi_A",
            "cell_volume", "row_ptr", "column_index")
    m = {k: setup[k] for k in keys}
    m.update(n_cells=setup["cell_volume"].size, n_faces=setup["face_left"].size,
             n_bc=setup["bc_left"].size)
    return m
