"""TEST INFRASTRUCTURE ONLY -- Python access to the CPU oracle.

Loads ``oracle/_build/libocsl_oracle.so`` (the C restatement of the reference's
linear-solve path, see ``ocsl_oracle.h``) and, where it was built from the
reference's own sources, ``oracle/_ref/liboracle_ref.so`` (the reference
itself behind a small C-ABI harness).  Only tests, the smoke check and the
CPU-baseline leg of the benchmark import this module; the product never does.

All matrices use the reference's CSR layout (``cmatrix_solver.h:33-51``):
``row_ptr`` and ``column_index`` as ``uint64`` (``size_t``) with the phantom
column ``2**64 - 1`` on boundary rows, ``value`` as ``float64``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libocsl_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "liboracle_ref.so")
REF_SHOCKTUBE = os.path.join(HERE, "_ref", "ref_shocktube")
# The reference's source directory: OCSL_REFERENCE_DIR, else a checkout named
# "reference" beside this repository.  Where neither exists, everything that
# needs the reference skips.
REF_DIR = os.environ.get("OCSL_REFERENCE_DIR") or os.path.normpath(
    os.path.join(HERE, "..", "..", "reference"))
PHANTOM = np.uint64(0xFFFFFFFFFFFFFFFF)

_P = C.c_void_p
_SZ = C.c_size_t


def reference_sources_present(reference_dir: str | None = None) -> bool:
    return os.path.isfile(os.path.join(reference_dir or REF_DIR, "cmatrix_solver.cpp"))


def build(reference_dir: str | None = None) -> None:
    """Compile the oracle (always) and the reference (when its sources exist)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    ref = reference_dir or REF_DIR
    if reference_sources_present(ref):
        subprocess.run(["make", "-s", "-C", HERE, "-j8", "ref", f"REF={ref}"], check=True)


def build_shim_drivers(reference_dir: str | None = None) -> dict:
    """Link the reference's own program with the C++ drop-in (oracle/Makefile
    ``shim``); returns the paths of the three drivers.  Needs the reference's
    sources and the built GPU library."""
    ref = reference_dir or REF_DIR
    subprocess.run(["make", "-s", "-C", HERE, "-j8", "shim", f"REF={ref}"], check=True)
    return {k: os.path.join(HERE, "_ref", f"ref_driver_{k}") for k in ("cpu", "fake", "gpu")}


def _ptr(a):
    return a.ctypes.data_as(_P) if a is not None else None


class _Lib:
    def __init__(self, path, protos):
        self.lib = C.CDLL(path)
        for name, (res, args) in protos.items():
            f = getattr(self.lib, name)
            f.restype = res
            f.argtypes = args


_CSR = [_SZ, _P, _P]
_ORACLE_PROTOS = {
    "orc_set_threads": (None, [C.c_int]),
    "orc_dot": (C.c_double, [_SZ, _P, _P]),
    "orc_dot_seq": (C.c_double, [_SZ, _P, _P]),
    "orc_gemv": (None, _CSR + [_P, _P, C.c_int, C.c_double, _P, _P]),
    "orc_extract_diag": (C.c_int, _CSR + [_P]),
    "orc_ilu_fixed_point": (None, _CSR + [_P, _P, C.c_int, _P]),
    "orc_forsub": (None, _CSR + [_P, _P, _P, _P]),
    "orc_backsub": (None, _CSR + [_P, _P, _P, _P]),
    "orc_cg_ref": (C.c_double, _CSR + [_P, _P, _P, _P]),
    "orc_bicgstab_ref": (C.c_double, _CSR + [_P, _P, _P, _P]),
    "orc_bicgstab_tol": (C.c_int, _CSR + [_P, _P, _P, C.c_double, C.c_int, C.c_int, _P, _P]),
    "orc_pcg_tol": (C.c_int, _CSR + [_P, _P, _P, C.c_double, C.c_int, _P, _P]),
    "orc_bicgstab_ir32": (C.c_int, _CSR + [_P, _P, _P, C.c_double, C.c_int, C.c_double,
                                           C.c_int, C.c_int, _P, _P, _P]),
    "orc_true_relres": (C.c_double, _CSR + [_P, _P, _P]),
    "orc_sum": (C.c_double, [_SZ, _P, C.c_int]),
    "orc_product": (None, [_SZ, _P, _P, _P]),
    "orc_axpy": (None, [_SZ, C.c_double, _P, C.c_double, _P, _P]),
    "orc_assemble": (None, _CSR + [C.c_int64, _P, _P, C.c_int64, _P, _P, _P, _P, _P, _P, _P,
                                   _P]),
    "orc_bc_value_grad": (None, [_SZ, _P, C.c_int64, _P, _P, _P, _P, _P]),
    "orc_flow_iterate": (C.c_int, _CSR + [C.c_int64, _P, _P, C.c_int64, _P, _P, _P, _P, _P, _P,
                                          _P, _P, _P, _P, _P, _P]),
    "orc_flow_iterate_with": (C.c_int, _CSR + [C.c_int64, _P, _P, C.c_int64, _P, _P, _P, _P,
                                               _P, _P, _P, _P]),
    "orc_flow_end_step": (None, [_SZ, _P]),
}
_REF_CSR = [_SZ, _SZ, _P, _P]
_REF_PROTOS = {
    "refh_set_threads": (None, [C.c_int]),
    "refh_cg_solve": (C.c_double, _REF_CSR + [_P, _P, _P]),
    "refh_bicgstab_solve": (C.c_double, _REF_CSR + [_P, _P, _P]),
    "refh_gemv": (None, _REF_CSR + [_P, C.c_double, _P, C.c_double, _P, _P]),
    "refh_norm": (C.c_double, [_SZ, _P, _P]),
    "refh_sum": (C.c_double, [_SZ, _P, C.c_int]),
    "refh_product": (None, [_SZ, _P, _P, _P]),
    "refh_axpy": (None, [_SZ, C.c_double, _P, C.c_double, _P, _P]),
    "refh_extract_diag": (None, _REF_CSR + [_P]),
    "refh_ilu_decompose": (None, _REF_CSR + [_P, _P]),
    "refh_forsub": (None, _REF_CSR + [_P, _P, _P]),
    "refh_backsub": (None, _REF_CSR + [_P, _P, _P]),
}


def _c64(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


class Oracle:
    """The C restatement.  Every method mirrors one reference function."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(f"oracle library missing: {path} (run oracle.build())")
        self._l = _Lib(path, _ORACLE_PROTOS).lib

    def set_threads(self, t: int) -> None:
        self._l.orc_set_threads(int(t))

    def dot(self, x, y):
        x, y = _c64(x), _c64(y)
        return self._l.orc_dot(x.size, _ptr(x), _ptr(y))

    def sum(self, x, absolute=False):
        """cmatrix_solver.cpp:244-263 sum / ABSsum in the tile order."""
        x = _c64(x)
        return self._l.orc_sum(x.size, _ptr(x), int(bool(absolute)))

    def product(self, x, y):
        x, y = _c64(x), _c64(y)
        out = np.zeros(x.size)
        self._l.orc_product(x.size, _ptr(x), _ptr(y), _ptr(out))
        return out

    def axpy(self, a, x, b=0.0, y=None):
        x = _c64(x)
        yy = None if y is None else _c64(y)
        out = np.zeros(x.size)
        self._l.orc_axpy(x.size, float(a), _ptr(x), float(b), _ptr(yy), _ptr(out))
        return out

    def dot_seq(self, x, y):
        x, y = _c64(x), _c64(y)
        return self._l.orc_dot_seq(x.size, _ptr(x), _ptr(y))

    @staticmethod
    def _csr(rp, col):
        return _c64(rp, np.uint64), _c64(col, np.uint64)

    def gemv(self, rp, col, val, x, mode=0, a=0.0, z=None):
        rp, col = self._csr(rp, col)
        n = rp.size - 1
        val, x = _c64(val), _c64(x)
        z = _c64(z) if z is not None else None
        y = np.zeros(n)
        self._l.orc_gemv(n, _ptr(rp), _ptr(col), _ptr(val), _ptr(x), mode, a, _ptr(z), _ptr(y))
        return y

    def extract_diag(self, rp, col):
        rp, col = self._csr(rp, col)
        d = np.zeros(rp.size - 1, np.int32)
        rc = self._l.orc_extract_diag(rp.size - 1, _ptr(rp), _ptr(col), _ptr(d))
        return d, rc

    def ilu(self, rp, col, A, sweeps=3):
        rp, col = self._csr(rp, col)
        d, _ = self.extract_diag(rp, col)
        A = _c64(A)
        M = np.zeros_like(A)
        self._l.orc_ilu_fixed_point(rp.size - 1, _ptr(rp), _ptr(col), _ptr(A), _ptr(d), sweeps,
                                    _ptr(M))
        return M

    def forsub(self, rp, col, M, b):
        rp, col = self._csr(rp, col)
        d, _ = self.extract_diag(rp, col)
        M, b = _c64(M), _c64(b)
        y = np.zeros(rp.size - 1)
        self._l.orc_forsub(rp.size - 1, _ptr(rp), _ptr(col), _ptr(M), _ptr(d), _ptr(b), _ptr(y))
        return y

    def backsub(self, rp, col, M, y):
        rp, col = self._csr(rp, col)
        d, _ = self.extract_diag(rp, col)
        M, y = _c64(M), _c64(y)
        x = np.zeros(rp.size - 1)
        self._l.orc_backsub(rp.size - 1, _ptr(rp), _ptr(col), _ptr(M), _ptr(d), _ptr(y), _ptr(x))
        return x

    def _solve_ref(self, fn, rp, col, val, b, x0):
        rp, col = self._csr(rp, col)
        val, b = _c64(val), _c64(b)
        x = _c64(x0).copy()
        it = C.c_int(0)
        res = fn(rp.size - 1, _ptr(rp), _ptr(col), _ptr(val), _ptr(b), _ptr(x), C.byref(it))
        return x, res, it.value

    def cg_ref(self, rp, col, val, b, x0):
        """cmatrix_solver.cpp:635 CG_solve -> (x, residual, iterations)."""
        return self._solve_ref(self._l.orc_cg_ref, rp, col, val, b, x0)

    def bicgstab_ref(self, rp, col, val, b, x0):
        """cmatrix_solver.cpp:682 ILU_BICGSTAB_solve -> (x, residual, iterations)."""
        return self._solve_ref(self._l.orc_bicgstab_ref, rp, col, val, b, x0)

    def bicgstab_tol(self, rp, col, val, b, x0, tol=1e-10, maxit=2000, sweeps=3):
        rp, col = self._csr(rp, col)
        val, b = _c64(val), _c64(b)
        x = _c64(x0).copy()
        it, rr = C.c_int(0), C.c_double(0)
        rc = self._l.orc_bicgstab_tol(rp.size - 1, _ptr(rp), _ptr(col), _ptr(val), _ptr(b),
                                      _ptr(x), tol, maxit, sweeps, C.byref(it), C.byref(rr))
        return x, rc, it.value, rr.value

    def pcg_tol(self, rp, col, val, b, x0, tol=1e-10, maxit=5000):
        rp, col = self._csr(rp, col)
        val, b = _c64(val), _c64(b)
        x = _c64(x0).copy()
        it, rr = C.c_int(0), C.c_double(0)
        rc = self._l.orc_pcg_tol(rp.size - 1, _ptr(rp), _ptr(col), _ptr(val), _ptr(b), _ptr(x),
                                 tol, maxit, C.byref(it), C.byref(rr))
        return x, rc, it.value, rr.value

    def bicgstab_ir32(self, rp, col, val, b, x0, tol=1e-10, maxit=2000, inner_tol=1e-5,
                      inner_maxit=200, sweeps=3):
        rp, col = self._csr(rp, col)
        val, b = _c64(val), _c64(b)
        x = _c64(x0).copy()
        it, out, rr = C.c_int(0), C.c_int(0), C.c_double(0)
        rc = self._l.orc_bicgstab_ir32(rp.size - 1, _ptr(rp), _ptr(col), _ptr(val), _ptr(b),
                                       _ptr(x), tol, maxit, inner_tol, inner_maxit, sweeps,
                                       C.byref(it), C.byref(out), C.byref(rr))
        return x, rc, it.value, out.value, rr.value

    def true_relres(self, rp, col, val, b, x):
        rp, col = self._csr(rp, col)
        val, b, x = _c64(val), _c64(b), _c64(x)
        return self._l.orc_true_relres(rp.size - 1, _ptr(rp), _ptr(col), _ptr(val), _ptr(b),
                                       _ptr(x))


def _assembly_struct(eq: dict):
    from opencslsolver_gb300 import _abi

    q = _abi.Assembly()
    for k in ("equation", "dimension", "viscous", "blended", "transient"):
        setattr(q, k, int(eq.get(k, 0)))
    for k in ("implicit_underrelaxation", "R_specific", "gamma", "prandtl"):
        setattr(q, k, float(eq.get(k, 0.0)))
    q.thermal_diffusivity = float(eq.get("thermal_diffusivity", 0.0))
    su = eq.get("sutherland", (0.0, 0.0))
    q.sutherland[0], q.sutherland[1] = float(su[0]), float(su[1])
    return q


def _host_state(state: dict):
    from opencslsolver_gb300 import _abi

    keep = {}
    for k, v in state.items():
        if v is None:
            continue
        dt = np.int32 if k in _abi.INT_FIELDS else np.float64
        keep[k] = np.ascontiguousarray(v, dtype=dt)
    return _abi.flow_state(keep, lambda a: a.ctypes.data), keep


def assemble(rp, col, left, right, bc_left, eq: dict, state: dict):
    """Oracle face-loop assembly (ocsl_oracle_assembly.c) -> value, b, x0, ap, total_mdot."""
    lib = Oracle()._l
    rp, col = np.ascontiguousarray(rp, np.uint64), np.ascontiguousarray(col, np.uint64)
    left, right = np.ascontiguousarray(left, np.int32), np.ascontiguousarray(right, np.int32)
    bc_left = np.ascontiguousarray(bc_left, np.int32)
    n = rp.size - 1
    q = _assembly_struct(eq)
    st, keep = _host_state(state)
    value, b, x0, ap, tm = (np.zeros(col.size), np.zeros(n), np.zeros(n), np.zeros(n),
                            np.zeros(n))
    lib.orc_assemble(n, _ptr(rp), _ptr(col), left.size, _ptr(left), _ptr(right), bc_left.size,
                     _ptr(bc_left), C.addressof(q), C.addressof(st), _ptr(value), _ptr(b),
                     _ptr(x0), _ptr(ap), _ptr(tm))
    del keep
    return value, b, x0, ap, tm


def bc_value_grad(rp, bc_left, eq: dict, state: dict, lam):
    lib = Oracle()._l
    rp = np.ascontiguousarray(rp, np.uint64)
    bc_left = np.ascontiguousarray(bc_left, np.int32)
    q = _assembly_struct(eq)
    st, keep = _host_state(state)
    lam = np.ascontiguousarray(lam, np.float64)
    g = np.zeros(bc_left.size)
    lib.orc_bc_value_grad(rp.size - 1, _ptr(rp), bc_left.size, _ptr(bc_left), C.addressof(q),
                          C.addressof(st), _ptr(lam), _ptr(g))
    del keep
    return g


def _flow_structs(case: dict):
    """The ocsl_flow_state / ocsl_flow_iteration of a flow case (dict with
    "state", "arrays", "constants"; arrays updated in place)."""
    from opencslsolver_gb300 import _abi

    for group in ("state", "arrays"):
        for k, v in case[group].items():
            dt = np.int32 if k in _abi.INT_FIELDS else np.float64
            if not (isinstance(v, np.ndarray) and v.dtype == dt and v.flags.c_contiguous):
                raise ValueError(f"{group}[{k}] must be a C-contiguous {np.dtype(dt)} array")
    st = _abi.flow_state(case["state"], lambda a: a.ctypes.data)
    it = _abi.flow_iteration(case["arrays"], case["constants"], lambda a: a.ctypes.data)
    return st, it


def flow_iterate(case: dict, methods, given_x=None, capture=False, tol=1e-10, maxit=5000,
                 ilu_sweeps=3):
    """One SIMPLE inner iteration of the oracle (ocsl_oracle_flow.c) on
    ``case`` (mesh, eq, state, arrays, constants), in place.  given_x: five
    solutions used instead of solving; tol / maxit / ilu_sweeps: the
    tolerance-mode methods' settings (the library's defaults).  Returns
    residuals[5], iterations[5] and, with capture, the five assembled systems
    (value, b, x0)."""
    from opencslsolver_gb300 import _abi
    lib = Oracle()._l
    rp = np.ascontiguousarray(case["row_ptr"], np.uint64)
    col = np.ascontiguousarray(case["column_index"], np.uint64)
    left = np.ascontiguousarray(case["left"], np.int32)
    right = np.ascontiguousarray(case["right"], np.int32)
    bc_left = np.ascontiguousarray(case["bc_left"], np.int32)
    n = rp.size - 1
    q = _assembly_struct(case["eq"])
    st, it = _flow_structs(case)
    m = (C.c_int * 3)(*[int(v) for v in methods])
    gx = None
    if given_x is not None:
        given = [np.ascontiguousarray(x, np.float64) for x in given_x]
        gx = (_P * 5)(*[_ptr(x) for x in given])
    sv = sb = sx = None
    if capture:
        sv, sb, sx = np.zeros((5, col.size)), np.zeros((5, n)), np.zeros((5, n))
    o = _abi.Opts()
    o.tol, o.maxit, o.ilu_sweeps = float(tol), int(maxit), int(ilu_sweeps)
    res, its = np.zeros(5), np.zeros(5, np.int32)
    rc = lib.orc_flow_iterate(n, _ptr(rp), _ptr(col), left.size, _ptr(left), _ptr(right),
                              bc_left.size, _ptr(bc_left), C.addressof(q), C.addressof(st),
                              C.addressof(it), m, C.addressof(o), gx, _ptr(sv), _ptr(sb),
                              _ptr(sx), _ptr(res), _ptr(its))
    if rc:
        raise ValueError("the oracle iteration supports CG_REF, BICGSTAB_REF, PCG and "
                         "ILU_BICGSTAB")
    out = {"residual": res, "iterations": its}
    if capture:
        out.update(value=sv, b=sb, x0=sx)
    return out


def flow_iterate_with(case: dict, methods, solve_fn) -> np.ndarray:
    """One SIMPLE inner iteration of the oracle on ``case`` with every solve
    handed to ``solve_fn``, a C function pointer of the orc_solve_fn type (an
    external solver under the oracle's host-side stages).  Returns the five
    residuals."""
    lib = Oracle()._l
    rp = np.ascontiguousarray(case["row_ptr"], np.uint64)
    col = np.ascontiguousarray(case["column_index"], np.uint64)
    left = np.ascontiguousarray(case["left"], np.int32)
    right = np.ascontiguousarray(case["right"], np.int32)
    bc_left = np.ascontiguousarray(case["bc_left"], np.int32)
    q = _assembly_struct(case["eq"])
    st, it = _flow_structs(case)
    m = (C.c_int * 3)(*[int(v) for v in methods])
    res = np.zeros(5)
    rc = lib.orc_flow_iterate_with(rp.size - 1, _ptr(rp), _ptr(col), left.size, _ptr(left),
                                   _ptr(right), bc_left.size, _ptr(bc_left), C.addressof(q),
                                   C.addressof(st), C.addressof(it), m,
                                   C.cast(solve_fn, _P), None, _ptr(res))
    if rc:
        raise RuntimeError("the external solver refused a solve")
    return res


def flow_end_step(case: dict) -> None:
    lib = Oracle()._l
    st, _ = _flow_structs(case)
    lib.orc_flow_end_step(np.asarray(case["row_ptr"]).size - 1, C.addressof(st))


def reference_available() -> bool:
    return os.path.isfile(REF_SO)


class Reference:
    """The reference's own CMatrix_solver, built from its sources (oracle/_ref)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.isfile(path):
            raise FileNotFoundError(f"reference harness missing: {path}")
        self._l = _Lib(path, _REF_PROTOS).lib
        self._l.refh_set_threads(1)

    def set_threads(self, t: int) -> None:
        self._l.refh_set_threads(int(t))

    @staticmethod
    def _args(rp, col):
        rp, col = _c64(rp, np.uint64), _c64(col, np.uint64)
        return rp, col, rp.size - 1, col.size

    def cg_solve(self, rp, col, val, b, x0):
        rp, col, n, nnz = self._args(rp, col)
        val, b, x = _c64(val), _c64(b), _c64(x0).copy()
        res = self._l.refh_cg_solve(n, nnz, _ptr(rp), _ptr(col), _ptr(val), _ptr(b), _ptr(x))
        return x, res

    def bicgstab_solve(self, rp, col, val, b, x0):
        rp, col, n, nnz = self._args(rp, col)
        val, b, x = _c64(val), _c64(b), _c64(x0).copy()
        res = self._l.refh_bicgstab_solve(n, nnz, _ptr(rp), _ptr(col), _ptr(val), _ptr(b),
                                          _ptr(x))
        return x, res

    def gemv(self, rp, col, val, a, x, bcoef=0.0, z=None):
        rp, col, n, nnz = self._args(rp, col)
        val, x = _c64(val), _c64(x)
        z = _c64(z) if z is not None else None
        y = np.zeros(n)
        self._l.refh_gemv(n, nnz, _ptr(rp), _ptr(col), _ptr(val), a, _ptr(x), bcoef, _ptr(z),
                          _ptr(y))
        return y

    def sum(self, x, absolute=False):
        x = _c64(x)
        return self._l.refh_sum(x.size, _ptr(x), int(bool(absolute)))

    def product(self, x, y):
        x, y = _c64(x), _c64(y)
        out = np.zeros(x.size)
        self._l.refh_product(x.size, _ptr(x), _ptr(y), _ptr(out))
        return out

    def axpy(self, a, x, b=0.0, y=None):
        x = _c64(x)
        yy = None if y is None else _c64(y)
        out = np.zeros(x.size)
        self._l.refh_axpy(x.size, float(a), _ptr(x), float(b), _ptr(yy), _ptr(out))
        return out

    def norm(self, x, y):
        x, y = _c64(x), _c64(y)
        return self._l.refh_norm(x.size, _ptr(x), _ptr(y))

    def extract_diag(self, rp, col):
        rp, col, n, nnz = self._args(rp, col)
        d = np.zeros(n, np.int32)
        self._l.refh_extract_diag(n, nnz, _ptr(rp), _ptr(col), _ptr(d))
        return d

    def ilu_decompose(self, rp, col, A):
        rp, col, n, nnz = self._args(rp, col)
        A = _c64(A)
        M = np.zeros_like(A)
        self._l.refh_ilu_decompose(n, nnz, _ptr(rp), _ptr(col), _ptr(A), _ptr(M))
        return M

    def forsub(self, rp, col, M, b):
        rp, col, n, nnz = self._args(rp, col)
        M, b = _c64(M), _c64(b)
        y = np.zeros(n)
        self._l.refh_forsub(n, nnz, _ptr(rp), _ptr(col), _ptr(M), _ptr(b), _ptr(y))
        return y

    def backsub(self, rp, col, M, y):
        rp, col, n, nnz = self._args(rp, col)
        M, y = _c64(M), _c64(y)
        x = np.zeros(n)
        self._l.refh_backsub(n, nnz, _ptr(rp), _ptr(col), _ptr(M), _ptr(y), _ptr(x))
        return x
