"""A SIMPLE run on the device from a mesh and a configuration.

``initial_state`` is the host-side set-up the reference does once in
CFlow_solver::initialize (cflow_solver.cpp:33-195): cells from the initial
condition (uniform, or the shock tube's two states), boundary faces from their
marker's boundary condition, ap = 1, and the first face and boundary mass
fluxes; ``FlowRun`` keeps the state on the device and runs inner iterations
(``ocsl_flow_iterate_device``) and time steps (``ocsl_flow_end_step_device``
plus the steady under-relaxation ramp of update_timestep,
cflow_solver.cpp:503-519).  With the mesh from ``read_su2`` and the pattern
from ``build_pattern`` nothing of the reference is needed at run time.

The set-up is numpy arithmetic; the reference's (compiled with -ffast-math)
differs in the last bits.  Every array of the state uses the names of
``ocsl_flow_state`` / ``ocsl_flow_iteration`` (include/ocsl.h); vectors are
[3][count].
"""
from __future__ import annotations

import numpy as np

from . import _abi

# Cfluid_properties defaults (cfluid_properties.h:38-50, cfluid_properties.cpp:30-38)
# and CFlow_solver's explicit under-relaxation (cflow_solver.h:178-179).
R_UNIVERSAL = 8.31446261815324
MOLAR_MASS_AIR = 28.9651159 / 1000.0
AIR = {"R_specific": R_UNIVERSAL / MOLAR_MASS_AIR, "gamma": 1.4, "Tref": 298.15,
       "H_formation": 0.0, "sutherland": (1.458e-6, 110.4), "prandtl": 0.713}
AIR["cp"] = (AIR["gamma"] * AIR["R_specific"]) / (AIR["gamma"] - 1.0)
RELAX_P, RELAX_U = 0.5, 0.8

KINDS = {"empty": _abi.BC_EMPTY, "symmetry": _abi.BC_SYMMETRY, "wall": _abi.BC_WALL,
         "velocity_inlet": _abi.BC_VELOCITY_INLET, "supersonic_inlet": _abi.BC_SUPERSONIC_INLET,
         "pressure_outlet": _abi.BC_PRESSURE_OUTLET}


def _dot(a, b):  # [3][count] component-major
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def _enthalpy(fl, T, u):  # cfluid_properties.cpp:98-106
    return fl["H_formation"] + (T - fl["Tref"]) * fl["cp"] + _dot(u, u) * 0.5


def _interp(blended, geo, m, l, r):  # solvers_common.h:69-90
    up = np.where(m >= 0.0, l, r)
    if not blended:
        return up
    return up * (1.0 - 0.7) + 0.7 * (geo * l + (1.0 - geo) * r)


def initial_state(mesh: dict, *, initial: dict, boundaries: list, viscous: bool = False,
                  blended: bool = True, transient: bool = True, dt: float = 1e-5,
                  implicit_underrelaxation: float = 0.5, ramp: tuple = (0.5, 0.8, 10.0),
                  fluid: dict = AIR) -> dict:
    """The state after CFlow_solver::initialize for ``mesh`` (the arrays of
    ``read_su2``, with ``row_ptr`` / ``column_index`` added).

    initial: {"pressure", "temperature", "velocity": (3,)} and for a shock tube
    also {"pressure2", "temperature2"} (cells from round(n/2) - 1 on,
    cflow_solver.cpp:58-72).  boundaries: one dict per mesh marker, in marker
    order: {"kind": "wall" | "empty" | "symmetry" | "velocity_inlet" |
    "supersonic_inlet" | "pressure_outlet", "velocity", "temperature",
    "pressure", "wall": "no_slip" | "slip", "thermal": "constant_temperature" |
    "adiabatic"}.  Returns a case dict with "state" and "arrays" (host numpy),
    "eq", "constants", the mesh connectivity and the ramp."""
    fl = fluid
    R = fl["R_specific"]
    n, nf, nb = int(mesh["n_cells"]), int(mesh["n_faces"]), int(mesh["n_bc"])
    L, Rt = mesh["face_left"].astype(np.int64), mesh["face_right"].astype(np.int64)
    bl = mesh["bc_left"].astype(np.int64)
    A = mesh["face_area_vector"].reshape(3, nf)
    bA = mesh["bc_area_vector"].reshape(3, nb)
    geo = mesh["face_geo_aver"]
    vol = mesh["cell_volume"]

    # cells (cflow_solver.cpp:40-72)
    p = np.full(n, float(initial["pressure"]))
    T = np.full(n, float(initial["temperature"]))
    u = np.repeat(np.asarray(initial["velocity"], float).reshape(3, 1), n, axis=1)
    if "pressure2" in initial:
        start = int(round(n // 2)) - 1
        p[start:] = initial["pressure2"]
        T[start:] = initial["temperature2"]
    rho = p / (R * T)
    h = _enthalpy(fl, T, u)

    # boundary faces (cflow_solver.cpp:88-150)
    kind = np.zeros(nb, np.int32)
    wall = np.zeros(nb, np.int32)
    thermal = np.zeros(nb, np.int32)
    sup = np.zeros(nb, np.int32)
    bp, bout, bT, bdens, bh, bm = (np.zeros(nb) for _ in range(6))
    bqy = np.ones(nb)  # CFlow_BC_face::Qy starts at 1 (cflow_solver.h:86)
    bV = np.zeros((3, nb))
    for mk, cfg in enumerate(boundaries):
        g = np.nonzero(mesh["bc_marker"] == mk)[0]
        k = KINDS[cfg["kind"]]
        kind[g] = k
        c = bl[g]
        if k in (_abi.BC_VELOCITY_INLET, _abi.BC_SUPERSONIC_INLET):
            V = np.asarray(cfg["velocity"], float).reshape(3, 1)
            bV[:, g] = V
            bT[g] = cfg["temperature"]
            bp[g] = p[c] if k == _abi.BC_VELOCITY_INLET else cfg["pressure"]
            bdens[g] = bp[g] / (R * bT[g])
            bh[g] = _enthalpy(fl, bT[g], bV[:, g])
            bm[g] = bdens[g] * _dot(bV[:, g], bA[:, g])
        elif k == _abi.BC_PRESSURE_OUTLET:
            bT[g] = T[c]
            bp[g] = cfg["pressure"]
            bout[g] = cfg["pressure"]
            bdens[g] = bp[g] / (R * bT[g])
            bV[:, g] = u[:, c]
            bm[g] = rho[c] * _dot(u[:, c], bA[:, g])
            bh[g] = _enthalpy(fl, T[c], u[:, c])
            fast = bm[g] / rho[c] / mesh["bc_area"][g] >= np.sqrt(R * T[c] * fl["gamma"])
            sup[g[fast]] = 1
            bp[g[fast]] = p[c[fast]]
            bdens[g[fast]] = bp[g[fast]] / (R * bT[g[fast]])
        elif k == _abi.BC_WALL:
            wall[g] = _abi.WALL_SLIP if cfg.get("wall", "no_slip") == "slip" else _abi.WALL_NO_SLIP
            thermal[g] = (_abi.THERMAL_ADIABATIC if cfg.get("thermal", "adiabatic") == "adiabatic"
                          else _abi.THERMAL_CONSTANT_TEMPERATURE)
            bp[g] = p[c]

    # ap = 1, the first face mass fluxes with a zero pressure gradient
    # (cflow_solver.cpp:152-176, cflow_solver_supply.cpp:25-93)
    ap = np.ones(n)
    alpha = mesh["face_alpha"].reshape(3, nf)
    qy = (vol[L] / ap[L] + vol[Rt] / ap[Rt]) * _dot(alpha, A)
    vf = geo * u[:, L] + (1.0 - geo) * u[:, Rt]
    m = _dot(vf, A) - qy * (p[Rt] - p[L])
    frho = _interp(blended, geo, m, rho[L], rho[Rt])
    m = m * frho
    balpha = mesh["bc_alpha"].reshape(3, nb)
    for g in np.nonzero(kind == _abi.BC_VELOCITY_INLET)[0]:
        c = bl[g]
        bm[g] = p[c] / (R * bT[g]) * _dot(bV[:, g], bA[:, g])
    for g in np.nonzero(kind == _abi.BC_SUPERSONIC_INLET)[0]:
        bqy[g] = vol[bl[g]] / ap[bl[g]] * _dot(balpha[:, g], bA[:, g])
    for g in np.nonzero(kind == _abi.BC_PRESSURE_OUTLET)[0]:
        c = bl[g]
        if sup[g]:
            bm[g] = p[c] / (R * T[c]) * _dot(u[:, c], bA[:, g])
            bqy[g] = 1.0
        else:
            q = vol[c] / ap[c] * _dot(balpha[:, g], bA[:, g])
            bqy[g] = q
            bm[g] = (_dot(u[:, c], bA[:, g]) - q * (bp[g] - p[c])) * bdens[g]

    z = lambda *shape: np.zeros(shape if len(shape) > 1 else shape[0])  # noqa: E731
    state = {
        "geo_aver": geo.copy(), "ksi_A": mesh["face_ksi_A"].copy(), "mdot": m, "density": frho,
        "qy": qy, "stress": z(3 * nf), "bc_type": kind, "bc_wall": wall, "bc_supersonic": sup,
        "bc_area": mesh["bc_area"].copy(), "bc_area_vector": mesh["bc_area_vector"].copy(),
        "bc_perp_dist": mesh["bc_perp_dist"].copy(), "bc_ksi_A": mesh["bc_ksi_A"].copy(),
        "bc_mdot": bm, "bc_density": bdens, "bc_qy": bqy, "bc_temperature": bT,
        "bc_enthalpy": bh, "bc_velocity": bV.reshape(-1), "volume": vol.copy(),
        # CFlow_cell::delta_t starts at 0.001 (cflow_solver.h:57); a transient run sets it
        "delta_t": np.full(n, float(dt) if transient else 0.001), "velocity": u.reshape(-1).copy(),
        "velocity_last": u.reshape(-1).copy(), "pressure_grad": z(3 * n), "density_c": rho,
        "density_last": rho.copy(), "pressure": p, "pressure_last": p.copy(),
        "pressure_corr": z(n), "temperature": T, "enthalpy": h, "enthalpy_last": h.copy(),
        "bc_thermal": thermal,
    }
    arrays = {
        "face_area_vector": mesh["face_area_vector"].copy(), "face_alpha": mesh["face_alpha"].copy(),
        "face_distance": mesh["face_distance"].copy(), "face_unit": mesh["face_unit"].copy(),
        "bc_distance": mesh["bc_distance"].copy(), "bc_unit": mesh["bc_unit"].copy(),
        "bc_alpha": mesh["bc_alpha"].copy(), "bc_out_pressure": bout, "bc_pressure": bp,
        "pressure_corr_grad": z(3 * n), "ap": ap, "ap_vec": z(3 * n), "mach": z(n),
        "total_mdot": z(n),
    }
    return {
        "row_ptr": mesh["row_ptr"], "column_index": mesh["column_index"], "left": mesh["face_left"],
        "right": mesh["face_right"], "bc_left": mesh["bc_left"], "bc_marker": mesh["bc_marker"],
        "eq": {"viscous": int(viscous), "blended": int(blended), "transient": int(transient),
               "R_specific": R, "gamma": fl["gamma"], "sutherland": fl["sutherland"],
               "prandtl": fl["prandtl"], "implicit_underrelaxation": implicit_underrelaxation},
        "constants": {"cp": fl["cp"], "Tref": fl["Tref"], "H_formation": fl["H_formation"],
                      "relax_p": RELAX_P, "relax_u": RELAX_U},
        "ramp": tuple(float(v) for v in ramp),
        "state": state, "arrays": arrays,
    }


class FlowRun:
    """A flow case (``initial_state`` or any dict of that shape) on the device:
    the pattern and faces bound to ``ctx``, every state array a CUDA tensor."""

    MAIN_FIELDS = ("pressure", "velocity", "temperature", "density_c", "enthalpy")

    def __init__(self, ctx, case: dict):
        import torch

        self.ctx = ctx
        self.case = case
        ctx.set_pattern(case["row_ptr"], case["column_index"])
        ctx.set_faces(case["left"], case["right"], case["bc_left"])

        def dev(k, v):
            dt = torch.int32 if k in _abi.INT_FIELDS else torch.float64
            return torch.from_numpy(np.ascontiguousarray(v)).to(device="cuda", dtype=dt)

        self.state = {k: dev(k, v) for k, v in case["state"].items()}
        self.arrays = {k: dev(k, v) for k, v in case["arrays"].items()}

    def iterate(self, methods, **opts) -> dict:
        """One inner iteration (CFlow_solver::iterate)."""
        return self.ctx.flow_iterate_device(self.case["eq"], self.state, self.arrays,
                                            self.case["constants"], methods, **opts)

    def end_step(self) -> None:
        """update_timestep: *_last = current, and the steady ramp."""
        self.ctx.flow_end_step_device(self.state)
        eq = self.case["eq"]
        init, top, steps = self.case["ramp"]
        if not eq["transient"] and eq["implicit_underrelaxation"] < top:
            eq["implicit_underrelaxation"] += (top - init) / steps

    def fields(self) -> dict:
        return {k: self.state[k].cpu().numpy() for k in self.MAIN_FIELDS}
