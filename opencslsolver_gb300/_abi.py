"""ctypes binding of the C ABI declared in include/ocsl.h.

Loads the in-tree ``_lib/libocsl_gb300.so``.  There is no fallback: if the
library is missing, importing the package still works (so the pure-host parts
and the docs stay usable), but every call that needs the library raises
``LibraryMissing``.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libocsl_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "ocsl.h")

OK, NOT_CONVERGED, ZERO_PIVOT, NONFINITE, BAD_PATTERN, TIMEOUT = 0, 1, 2, 3, 4, 5
CUDA_ERROR, BAD_ARGUMENT, NO_PATTERN, NO_DEVICE, BREAKDOWN = 6, 7, 8, 9, 10

CG_REF, BICGSTAB_REF, PCG, ILU_BICGSTAB, ILU_BICGSTAB_IR32 = 0, 1, 2, 3, 4
METHODS = {
    "cg_ref": CG_REF,
    "bicgstab_ref": BICGSTAB_REF,
    "pcg": PCG,
    "ilu_bicgstab": ILU_BICGSTAB,
    "ilu_bicgstab_ir32": ILU_BICGSTAB_IR32,
}


class LibraryMissing(RuntimeError):
    pass


class OcslError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class Opts(C.Structure):
    _fields_ = [("tol", C.c_double), ("maxit", C.c_int), ("ilu_sweeps", C.c_int),
                ("inner_tol", C.c_double), ("inner_maxit", C.c_int)]


class Result(C.Structure):
    _fields_ = [("residual", C.c_double), ("iterations", C.c_int),
                ("outer_iterations", C.c_int), ("status", C.c_int), ("solve_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = C.c_void_p
_SZ = C.c_size_t

# ocsl_assembly / ocsl_flow_state (include/ocsl.h), in declaration order.
EQ_MOMENTUM, EQ_PRESSURE, EQ_ENTHALPY, EQ_HEAT = 0, 1, 2, 3
THERMAL_CONSTANT_TEMPERATURE, THERMAL_ADIABATIC = 0, 1
BC_EMPTY, BC_SYMMETRY, BC_WALL, BC_VELOCITY_INLET, BC_SUPERSONIC_INLET, BC_PRESSURE_OUTLET = range(6)
WALL_NO_SLIP, WALL_SLIP = 0, 1


class Assembly(C.Structure):
    _fields_ = [("equation", C.c_int), ("dimension", C.c_int), ("viscous", C.c_int),
                ("blended", C.c_int), ("transient", C.c_int),
                ("implicit_underrelaxation", C.c_double), ("R_specific", C.c_double),
                ("gamma", C.c_double), ("sutherland", C.c_double * 2), ("prandtl", C.c_double),
                ("thermal_diffusivity", C.c_double)]


FLOW_STATE_FIELDS = (
    "geo_aver", "ksi_A", "mdot", "density", "qy", "stress",
    "bc_type", "bc_wall", "bc_supersonic", "bc_area", "bc_area_vector", "bc_perp_dist",
    "bc_ksi_A", "bc_mdot", "bc_density", "bc_qy", "bc_temperature", "bc_enthalpy",
    "bc_velocity", "bc_value",
    "volume", "delta_t", "velocity", "velocity_last", "pressure_grad", "density_c",
    "density_last", "pressure", "pressure_last", "pressure_corr", "temperature", "enthalpy",
    "enthalpy_last", "bc_thermal")
INT_FIELDS = ("bc_type", "bc_wall", "bc_supersonic", "bc_thermal")


class BatchSystem(C.Structure):
    _fields_ = [("n", C.c_size_t), ("row_ptr", C.c_void_p), ("column_index", C.c_void_p),
                ("nrhs", C.c_int)]


class FlowState(C.Structure):
    _fields_ = [(f, C.c_void_p) for f in FLOW_STATE_FIELDS]


def flow_state(arrays: dict, ptr) -> FlowState:
    """FlowState from named arrays; ``ptr(a)`` gives each array's address
    (host numpy or device tensor); missing names are NULL."""
    st = FlowState()
    for f in FLOW_STATE_FIELDS:
        a = arrays.get(f)
        setattr(st, f, None if a is None else ptr(a))
    return st

# ocsl_flow_iteration / ocsl_flow_report (include/ocsl.h)
FLOW_ITERATION_ARRAYS = (
    "face_area_vector", "face_alpha", "face_distance", "face_unit", "bc_distance", "bc_unit",
    "bc_alpha", "bc_out_pressure", "bc_pressure", "pressure_corr_grad", "ap", "ap_vec", "mach",
    "total_mdot")
FLOW_ITERATION_CONSTANTS = ("cp", "Tref", "H_formation", "relax_p", "relax_u")


class FlowIteration(C.Structure):
    _fields_ = ([(f, C.c_void_p) for f in FLOW_ITERATION_ARRAYS] +
                [(f, C.c_double) for f in FLOW_ITERATION_CONSTANTS])


class FlowReport(C.Structure):
    _fields_ = [("residual", C.c_double * 5), ("iterations", C.c_int * 5),
                ("status", C.c_int * 5)]

    def as_dict(self) -> dict:
        return {"residual": list(self.residual), "iterations": list(self.iterations),
                "status": list(self.status)}


def flow_iteration(arrays: dict, constants: dict, ptr) -> FlowIteration:
    """FlowIteration from named arrays (``ptr(a)`` gives each address) and the
    five constants; missing arrays are NULL."""
    it = FlowIteration()
    for f in FLOW_ITERATION_ARRAYS:
        a = arrays.get(f)
        setattr(it, f, None if a is None else ptr(a))
    for f in FLOW_ITERATION_CONSTANTS:
        setattr(it, f, float(constants[f]))
    return it


# ocsl_mesh_arrays (include/ocsl.h), in declaration order
MESH_ARRAYS = (
    ("face_left", "i", 1, "n_faces"), ("face_right", "i", 1, "n_faces"),
    ("face_geo_aver", "d", 1, "n_faces"), ("face_ksi_A", "d", 1, "n_faces"),
    ("face_area_vector", "d", 3, "n_faces"), ("face_alpha", "d", 3, "n_faces"),
    ("face_distance", "d", 1, "n_faces"), ("face_unit", "d", 3, "n_faces"),
    ("bc_left", "i", 1, "n_bc"), ("bc_marker", "i", 1, "n_bc"), ("bc_area", "d", 1, "n_bc"),
    ("bc_area_vector", "d", 3, "n_bc"), ("bc_alpha", "d", 3, "n_bc"),
    ("bc_distance", "d", 1, "n_bc"), ("bc_unit", "d", 3, "n_bc"),
    ("bc_perp_dist", "d", 1, "n_bc"), ("bc_ksi_A", "d", 1, "n_bc"),
    ("cell_volume", "d", 1, "n_cells"), ("cell_center", "d", 3, "n_cells"))


class VtkFields(C.Structure):
    """ocsl_vtk_fields (include/ocsl.h)."""
    _fields_ = [("heat", C.c_int), ("digits", C.c_int), ("density", C.c_void_p),
                ("pressure", C.c_void_p), ("temperature", C.c_void_p), ("mach", C.c_void_p),
                ("velocity", C.c_void_p), ("pressure_grad", C.c_void_p),
                ("bc_temperature", C.c_void_p), ("bc_type", C.c_void_p), ("bc_wall", C.c_void_p),
                ("viscous", C.c_int), ("sutherland", C.c_double * 2)]


class MeshArrays(C.Structure):
    _fields_ = ([("n_cells", C.c_int64), ("n_faces", C.c_int64), ("n_bc", C.c_int64),
                 ("n_markers", C.c_int32)] +
                [(name, C.POINTER(C.c_int32) if kind == "i" else C.POINTER(C.c_double))
                 for name, kind, _, _ in MESH_ARRAYS])


_CTX = C.c_void_p
_PROTOS = {
    "ocsl_default_opts": (None, [C.POINTER(Opts)]),
    "ocsl_status_string": (C.c_char_p, [C.c_int]),
    "ocsl_last_error": (C.c_char_p, [_CTX]),
    "ocsl_version": (C.c_char_p, []),
    "ocsl_create": (C.c_int, [C.POINTER(_CTX), C.c_int]),
    "ocsl_destroy": (C.c_int, [_CTX]),
    "ocsl_set_stream": (C.c_int, [_CTX, _P]),
    "ocsl_synchronize": (C.c_int, [_CTX]),
    "ocsl_set_pattern": (C.c_int, [_CTX, _SZ, _P, _P]),
    "ocsl_check_pattern": (C.c_int, [_SZ, _P, _P, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_char_p,
                                     _SZ]),
    "ocsl_build_pattern": (C.c_int, [_SZ, C.c_int64, _P, _P, C.c_int64, _P, _P, _P,
                                     C.POINTER(_SZ)]),
    "ocsl_pattern_info": (C.c_int, [_CTX, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                    C.POINTER(C.c_int32)]),
    "ocsl_solve": (C.c_int, [_CTX, C.c_int, _P, _P, _P, C.POINTER(Opts), C.POINTER(Result)]),
    "ocsl_solve_device": (C.c_int, [_CTX, C.c_int, _P, _P, _P, C.POINTER(Opts),
                                    C.POINTER(Result)]),
    "ocsl_solve_multi_device": (C.c_int, [_CTX, C.c_int, _P, C.c_int, _P, _P, C.POINTER(Opts),
                                          C.POINTER(Result)]),
    "ocsl_batch_create": (C.c_int, [C.POINTER(_P), C.c_int, C.c_int, C.POINTER(BatchSystem),
                                    C.c_int]),
    "ocsl_batch_destroy": (C.c_int, [_P]),
    "ocsl_batch_solve_device": (C.c_int, [_P, C.c_int, C.POINTER(_P), C.POINTER(_P),
                                          C.POINTER(_P), C.POINTER(Opts), C.POINTER(Result)]),
    "ocsl_batch_last_error": (C.c_char_p, [_P]),
    "ocsl_gemv_device": (C.c_int, [_CTX, C.c_int, C.c_double, _P, _P, _P, _P]),
    "ocsl_dot_device": (C.c_int, [_CTX, _SZ, _P, _P, C.POINTER(C.c_double)]),
    "ocsl_sum_device": (C.c_int, [_CTX, _SZ, _P, C.c_int, C.POINTER(C.c_double)]),
    "ocsl_product_device": (C.c_int, [_CTX, _SZ, _P, _P, _P]),
    "ocsl_axpy_device": (C.c_int, [_CTX, _SZ, C.c_double, _P, C.c_double, _P, _P]),
    "ocsl_ilu_device": (C.c_int, [_CTX, _P, _P, C.c_int]),
    "ocsl_forsub_device": (C.c_int, [_CTX, _P, _P, _P]),
    "ocsl_backsub_device": (C.c_int, [_CTX, _P, _P, _P]),
    "ocsl_solve_transpose": (C.c_int, [_CTX, C.c_int, _P, _P, _P, C.POINTER(Opts),
                                       C.POINTER(Result)]),
    "ocsl_solve_transpose_device": (C.c_int, [_CTX, C.c_int, _P, _P, _P, C.POINTER(Opts),
                                              C.POINTER(Result)]),
    "ocsl_pattern_outer_device": (C.c_int, [_CTX, C.c_double, _P, _P, _P]),
    "ocsl_set_faces": (C.c_int, [_CTX, C.c_int64, _P, _P, C.c_int64, _P]),
    "ocsl_assemble_device": (C.c_int, [_CTX, C.POINTER(Assembly), C.POINTER(FlowState), _P, _P,
                                       _P, _P, _P]),
    "ocsl_bc_value_grad_device": (C.c_int, [_CTX, C.POINTER(Assembly), C.POINTER(FlowState), _P,
                                            _P]),
    "ocsl_flow_iterate_device": (C.c_int, [_CTX, C.POINTER(Assembly), C.POINTER(FlowState),
                                           C.POINTER(FlowIteration), C.POINTER(C.c_int),
                                           C.POINTER(Opts), C.POINTER(FlowReport)]),
    "ocsl_flow_end_step_device": (C.c_int, [_CTX, C.POINTER(FlowState)]),
    "ocsl_mesh_read_su2": (C.c_int, [C.c_char_p, C.POINTER(_P), C.c_char_p, _SZ]),
    "ocsl_mesh_view": (C.c_int, [_P, C.POINTER(MeshArrays)]),
    "ocsl_mesh_marker_name": (C.c_char_p, [_P, C.c_int]),
    "ocsl_mesh_destroy": (C.c_int, [_P]),
    "ocsl_set_device_loop": (C.c_int, [_P, C.c_int]),
    "ocsl_batch_set_graph": (C.c_int, [_P, C.c_int]),
    "ocsl_set_spmv_lanes": (C.c_int, [_P, C.c_int]),
    "ocsl_spmv_lanes": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "ocsl_autotune_spmv_device": (C.c_int, [_P, C.c_int, _P, C.POINTER(C.c_int),
                                            C.POINTER(C.c_double)]),
    "ocsl_vtk_write": (C.c_int, [_P, C.POINTER(VtkFields), C.c_char_p, C.c_char_p, C.c_char_p,
                                 _SZ]),
    "ocsl_set_sweep_kernel": (C.c_int, [_CTX, C.c_int, C.c_int, C.c_int]),
    "ocsl_sweep_info": (C.c_int, [_CTX, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int)]),
    "ocsl_set_sweep_cluster": (C.c_int, [_CTX, C.c_int, C.c_int]),
    "ocsl_sweep_geometry": (C.c_int, [_CTX, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ocsl_wave_geometry": (C.c_int, [_CTX, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int)]),
    "ocsl_dot_noalloc": (C.c_int, [_SZ, _P, _P, _P, _P]),
    "ocsl_noalloc_last_error": (C.c_char_p, []),
    "ocsl_set_graphs": (C.c_int, [_CTX, C.c_int]),
    "ocsl_inject_fault": (C.c_int, [_CTX, C.c_int]),
    "ocsl_set_col_batching": (C.c_int, [_CTX, C.c_int]),
    "ocsl_set_ordering": (C.c_int, [_CTX, C.c_int]),
    "ocsl_ordering_info": (C.c_int, [_CTX, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                     C.POINTER(C.c_int32), C.POINTER(C.c_int)]),
    "ocsl_ordering_permutation": (C.c_int, [_CTX, C.POINTER(C.c_int32), _SZ]),
    "ocsl_colour_pattern": (C.c_int, [_SZ, _P, _P, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                      C.c_char_p, _SZ]),
    "ocsl_autotune_device": (C.c_int, [_CTX, C.c_int, C.c_void_p, C.POINTER(C.c_int),
                                       C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "ocsl_profile_enable": (C.c_int, [_CTX, C.c_int]),
    "ocsl_profile_read": (C.c_int, [_CTX, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "ocsl_profile_category_name": (C.c_char_p, [C.c_int]),
}
PROFILE_CATEGORIES = 10
ORDER_NATURAL, ORDER_MULTICOLOUR = 0, 1

_lib = None


def header_symbols() -> list[str]:
    """Names of every function include/ocsl.h declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ocsl_[a-z_0-9]+)\s*\(", text)))


def lib():
    """The loaded C library (raises LibraryMissing when it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise LibraryMissing(f"{LIB_PATH} is missing: run opencslsolver_gb300.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _PROTOS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(s: int) -> str:
    return lib().ocsl_status_string(int(s)).decode()


def default_opts(**kw) -> Opts:
    o = Opts()
    lib().ocsl_default_opts(C.byref(o))
    for k, v in kw.items():
        if v is not None:
            setattr(o, k, v)
    return o
