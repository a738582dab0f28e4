"""Loads the recorded face-loop assembly cases (tests/golden/assembly_*.npz,
made by tests/golden/make_golden.py from the reference) into the argument
form of the oracle's and the library's assembly entry points."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ("shocktube", "channel", "steady", "heat")
EQUATIONS = ("momentum_x", "momentum_y", "momentum_z", "pressure", "enthalpy", "heat")

# state field of the C ABI <- recorded array name
STATE_MAP = {
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


class Call:
    def __init__(self, z, k):
        g = lambda key: z[key] if key in z.files else z[f"c{k}_{key}"]
        self.row_ptr, self.column_index = z["row_ptr"], z["column_index"]
        self.left, self.right, self.bc_left = z["face_left"], z["face_right"], z["bc_left"]
        meta, fluid = g("meta"), g("fluid")
        eq = int(meta[0])
        self.name = EQUATIONS[eq]
        self.n = self.row_ptr.size - 1
        has = lambda key: key in z.files or f"c{k}_{key}" in z.files
        if self.name == "heat":
            self.eq = {"equation": 3, "transient": 1, "thermal_diffusivity": fluid[6]}
            self.state = {k_: g(v) for k_, v in STATE_MAP.items() if has(v)}
            self.state["delta_t"] = np.full(self.n, fluid[7])
            self.ap_vec = self.total_mdot = None
        else:
            self.eq = {
                "equation": 0 if eq < 3 else (1 if eq == 3 else 2),
                "dimension": eq if eq < 3 else 0,
                "viscous": int(meta[1]), "blended": int(meta[2]), "transient": int(meta[3]),
                "R_specific": fluid[0], "gamma": fluid[1], "sutherland": (fluid[2], fluid[3]),
                "prandtl": fluid[4], "implicit_underrelaxation": fluid[5],
            }
            self.state = {k_: g(v) for k_, v in STATE_MAP.items()}
            self.ap_vec, self.total_mdot = g("cell_ap_vec"), g("cell_total_mdot")
        self.value, self.b, self.x0 = g("value"), g("b"), g("x0")

    @property
    def ap_expected(self):
        d = self.eq["dimension"]
        return self.ap_vec.reshape(3, self.n)[d]


def load(case):
    z = np.load(os.path.join(GOLDEN, f"assembly_{case}.npz"), allow_pickle=False)
    return [Call(z, k) for k in range(int(z["count"]))]


def to_device(torch, state):
    """Assembly state dict -> CUDA tensors (int32 for the boundary kinds)."""
    from opencslsolver_gb300 import _abi

    out = {}
    for k, v in state.items():
        if v is None:
            continue
        dt = torch.int32 if k in _abi.INT_FIELDS else torch.float64
        out[k] = torch.as_tensor(np.ascontiguousarray(v)).to(device="cuda", dtype=dt).contiguous()
    return out
