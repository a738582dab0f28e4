"""GB300-native replacement of OpenCSLSolver's linear-solve hot path.

The product is the C-ABI library ``_lib/libocsl_gb300.so`` (include/ocsl.h),
hand-written sm_103a kernels behind ``extern "C"`` entry points.  This module
is the Python host side above that boundary:

* ``Context``: one device context with a fixed CSR pattern (host arrays in the
  reference layout, or device tensors for the resident-data entry points);
* ``CMatrix_solver``: a mirror of the reference class (``cmatrix_solver.h:27-95``)
  with the same members (``matrix`` with ``value``/``row_ptr``/``column_index``,
  ``b_vector``, ``x_vector``) and entry points (``CG_solve``,
  ``ILU_BICGSTAB_solve``, ``solve``), so code written against the reference
  reads the same.

Nothing here computes on the CPU: every numerical call goes through the CUDA
library and fails loudly (``LibraryMissing`` / ``OcslError``) without it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi
from ._abi import (BICGSTAB_REF, CG_REF, ILU_BICGSTAB, ILU_BICGSTAB_IR32, METHODS, PCG,
                   LibraryMissing, OcslError, Opts, Result)

PHANTOM = np.uint64(0xFFFFFFFFFFFFFFFF)

__all__ = ["Context", "Batch", "CMatrix_solver", "build_pattern", "check_pattern", "colour_pattern",
           "read_su2", "Mesh",
           "LibraryMissing", "OcslError",
           "CG_REF", "BICGSTAB_REF", "PCG", "ILU_BICGSTAB", "ILU_BICGSTAB_IR32", "METHODS",
           "PHANTOM"]


def _method(m) -> int:
    if isinstance(m, str):
        return METHODS[m]
    return int(m)


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def _dptr(t):
    """Device pointer of a CUDA tensor (torch) or an integer address."""
    if t is None:
        return None
    if isinstance(t, int):
        return C.c_void_p(t)
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("device entry points take contiguous CUDA tensors")
    return C.c_void_p(t.data_ptr())


def check_pattern(row_ptr, column_index):
    """Host-only validation + level analysis (ocsl_check_pattern).

    Returns ``(status, info)`` with ``info = {"nnz_real", "fw_levels",
    "bw_levels", "box", "error"}``; ``box`` is the detected 7-point box
    ``(nx, ny, nz)`` or zeros.
    """
    rp, col = _u64(row_ptr), _u64(column_index)
    nr, fw, bw = C.c_int64(0), C.c_int32(0), C.c_int32(0)
    box = (C.c_int32 * 3)()
    buf = C.create_string_buffer(512)
    st = _abi.lib().ocsl_check_pattern(rp.size - 1, _ptr(rp), _ptr(col), C.byref(nr),
                                       C.byref(fw), C.byref(bw), box, buf, 512)
    return st, {"nnz_real": nr.value, "fw_levels": fw.value, "bw_levels": bw.value,
                "box": tuple(box), "error": buf.value.decode()}


def colour_pattern(row_ptr, column_index):
    """Host-only multicolour ordering (ocsl_colour_pattern): ``(status,
    perm, colours, error)`` with perm[new row] = original row (int32)."""
    rp, col = _u64(row_ptr), _u64(column_index)
    n = rp.size - 1
    perm = np.zeros(max(n, 0), dtype=np.int32)
    k = C.c_int32(0)
    buf = C.create_string_buffer(512)
    st = _abi.lib().ocsl_colour_pattern(n, _ptr(rp), _ptr(col),
                                        perm.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(k),
                                        buf, 512)
    return st, perm, k.value, buf.value.decode()


class Context:
    """One GPU context (ocsl_create) holding one fixed CSR pattern."""

    def __init__(self, device: int = 0):
        self._L = _abi.lib()
        h = C.c_void_p()
        st = self._L.ocsl_create(C.byref(h), int(device))
        if st != 0:
            raise OcslError(st, self._L.ocsl_last_error(None).decode())
        self._h = h
        self.n = None
        self.nnz = None
        self._explicit_stream = False

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._L.ocsl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st, what):
        if st not in (0,):
            raise OcslError(st, f"{what}: {self._L.ocsl_status_string(st).decode()}: "
                                f"{self._L.ocsl_last_error(self._h).decode()}")

    def set_stream(self, stream_handle: int | None):
        """Run on a caller-owned cudaStream_t (None: back to following torch's
        current stream for the device entry points)."""
        self._explicit_stream = stream_handle is not None
        self._check(self._L.ocsl_set_stream(self._h, C.c_void_p(stream_handle or 0)),
                    "set_stream")

    def _follow_torch(self):
        """Device entry points run on torch's current stream unless a stream
        was set explicitly, so they are ordered after the torch work that
        produced their inputs (the legacy default stream is passed as
        cudaStreamLegacy)."""
        if self._explicit_stream:
            return
        import torch

        h = torch.cuda.current_stream().cuda_stream
        self._L.ocsl_set_stream(self._h, C.c_void_p(h if h else 1))

    def synchronize(self):
        self._check(self._L.ocsl_synchronize(self._h), "synchronize")

    # -- pattern (CFVM::define_matrix_structure, cfvm.cpp:74-98)
    def set_pattern(self, row_ptr, column_index):
        rp, col = _u64(row_ptr), _u64(column_index)
        st = self._L.ocsl_set_pattern(self._h, rp.size - 1, _ptr(rp), _ptr(col))
        self._check(st, "set_pattern")
        self.n, self.nnz = rp.size - 1, col.size
        return self

    def pattern_info(self):
        n, nnz, nr = C.c_int64(), C.c_int64(), C.c_int64()
        fw, bw = C.c_int32(), C.c_int32()
        self._check(self._L.ocsl_pattern_info(self._h, C.byref(n), C.byref(nnz), C.byref(nr),
                                              C.byref(fw), C.byref(bw)), "pattern_info")
        return {"n": n.value, "nnz": nnz.value, "nnz_real": nr.value, "fw_levels": fw.value,
                "bw_levels": bw.value}

    # -- solves
    def solve(self, method, value, b, x, *, raise_on_status=False, **opts):
        """Host-buffer solve (ocsl_solve).  ``x`` (float64 numpy) is updated in
        place, as the reference overwrites x_vector.  Returns a result dict
        with ``status``; ``raise_on_status`` turns non-OK statuses into errors."""
        val, bb = _f64(value), _f64(b)
        if not (isinstance(x, np.ndarray) and x.dtype == np.float64 and x.flags.c_contiguous):
            raise ValueError("x must be a C-contiguous float64 numpy array (updated in place)")
        o = _abi.default_opts(**opts)
        r = Result()
        st = self._L.ocsl_solve(self._h, _method(method), _ptr(val), _ptr(bb), _ptr(x),
                                C.byref(o), C.byref(r))
        if st in (_abi.CUDA_ERROR, _abi.BAD_ARGUMENT, _abi.NO_PATTERN) or (raise_on_status and st):
            self._check(st, "solve")
        return r.as_dict()

    def solve_device(self, method, value, b, x, *, raise_on_status=False, **opts):
        """Resident-data solve (ocsl_solve_device) on CUDA tensors; x in/out."""
        self._follow_torch()
        o = _abi.default_opts(**opts)
        r = Result()
        st = self._L.ocsl_solve_device(self._h, _method(method), _dptr(value), _dptr(b), _dptr(x),
                                       C.byref(o), C.byref(r))
        if st in (_abi.CUDA_ERROR, _abi.BAD_ARGUMENT, _abi.NO_PATTERN) or (raise_on_status and st):
            self._check(st, "solve_device")
        return r.as_dict()

    # -- face-loop assembly (cflow_solver_cell_face_loops.cpp)
    def set_faces(self, left, right, bc_left):
        """Mesh face connectivity (interior faces: left/right cells; boundary
        faces: their cell), once per mesh after set_pattern."""
        l = np.ascontiguousarray(left, dtype=np.int32)
        r = np.ascontiguousarray(right, dtype=np.int32)
        bl = np.ascontiguousarray(bc_left, dtype=np.int32)
        self._check(self._L.ocsl_set_faces(self._h, l.size, _ptr(l), _ptr(r), bl.size, _ptr(bl)),
                    "set_faces")

    @staticmethod
    def _assembly(eq: dict):
        q = _abi.Assembly()
        for k in ("equation", "dimension", "viscous", "blended", "transient"):
            setattr(q, k, int(eq.get(k, 0)))
        for k in ("implicit_underrelaxation", "R_specific", "gamma", "prandtl"):
            setattr(q, k, float(eq.get(k, 0.0)))
        q.thermal_diffusivity = float(eq.get("thermal_diffusivity", 0.0))
        q.sutherland[0], q.sutherland[1] = (float(v) for v in eq.get("sutherland", (0.0, 0.0)))
        return q

    def assemble_device(self, eq: dict, state: dict, value, b, x0, ap=None, total_mdot=None):
        """Assemble one equation on the device.  ``state`` maps the fields of
        ocsl_flow_state to CUDA tensors (float64; bc_type, bc_wall,
        bc_supersonic int32); outputs are CUDA float64 tensors."""
        self._follow_torch()
        q = self._assembly(eq)
        st = _abi.flow_state(state, lambda t: _dptr(t).value)
        self._check(self._L.ocsl_assemble_device(self._h, C.byref(q), C.byref(st), _dptr(value),
                                                 _dptr(b), _dptr(x0), _dptr(ap),
                                                 _dptr(total_mdot)), "assemble")

    def bc_value_grad_device(self, eq: dict, state: dict, lam, grad):
        """grad[g] = lam[cell of g] * D_g for the Dirichlet p' boundary faces."""
        self._follow_torch()
        q = self._assembly(eq)
        st = _abi.flow_state(state, lambda t: _dptr(t).value)
        self._check(self._L.ocsl_bc_value_grad_device(self._h, C.byref(q), C.byref(st),
                                                      _dptr(lam), _dptr(grad)), "bc_value_grad")

    def flow_iterate_device(self, eq: dict, state: dict, arrays: dict, constants: dict,
                            methods=(CG_REF, BICGSTAB_REF, BICGSTAB_REF), **opts) -> dict:
        """One SIMPLE inner iteration on the device (ocsl_flow_iterate_device).
        ``state`` maps ocsl_flow_state fields to CUDA tensors, updated in place;
        ``arrays`` the device arrays of ocsl_flow_iteration (metrics and the
        fields the iteration writes), ``constants`` its cp, Tref, H_formation,
        relax_p, relax_u.  Returns the report; a failing solve raises."""
        self._follow_torch()
        q = self._assembly(eq)
        st = _abi.flow_state(state, lambda t: _dptr(t).value)
        it = _abi.flow_iteration(arrays, constants, lambda t: _dptr(t).value)
        m = (C.c_int * 3)(*(_method(x) for x in methods))
        o = _abi.default_opts(**opts)
        rep = _abi.FlowReport()
        self._check(self._L.ocsl_flow_iterate_device(self._h, C.byref(q), C.byref(st),
                                                     C.byref(it), m, C.byref(o), C.byref(rep)),
                    "flow_iterate")
        return rep.as_dict()

    def flow_end_step_device(self, state: dict) -> None:
        """Copy velocity, density, pressure and enthalpy to their *_last fields."""
        self._follow_torch()
        st = _abi.flow_state(state, lambda t: _dptr(t).value)
        self._check(self._L.ocsl_flow_end_step_device(self._h, C.byref(st)), "flow_end_step")

    # -- adjoint (no reference counterpart)
    def solve_transpose(self, method, value, g, lam, *, raise_on_status=False, **opts):
        """Host-buffer adjoint solve A^T lam = g (ocsl_solve_transpose); ``value``
        holds A in A's own CSR order, ``lam`` (float64 numpy) is in/out."""
        val, gg = _f64(value), _f64(g)
        if not (isinstance(lam, np.ndarray) and lam.dtype == np.float64 and lam.flags.c_contiguous):
            raise ValueError("lam must be a C-contiguous float64 numpy array (updated in place)")
        o = _abi.default_opts(**opts)
        r = Result()
        st = self._L.ocsl_solve_transpose(self._h, _method(method), _ptr(val), _ptr(gg), _ptr(lam),
                                          C.byref(o), C.byref(r))
        if st in (_abi.CUDA_ERROR, _abi.BAD_ARGUMENT, _abi.NO_PATTERN, _abi.BAD_PATTERN) or (
                raise_on_status and st):
            self._check(st, "solve_transpose")
        return r.as_dict()

    def solve_transpose_device(self, method, value, g, lam, *, raise_on_status=False, **opts):
        """Resident-data adjoint solve A^T lam = g on CUDA tensors; lam in/out."""
        self._follow_torch()
        o = _abi.default_opts(**opts)
        r = Result()
        st = self._L.ocsl_solve_transpose_device(self._h, _method(method), _dptr(value), _dptr(g),
                                                 _dptr(lam), C.byref(o), C.byref(r))
        if st in (_abi.CUDA_ERROR, _abi.BAD_ARGUMENT, _abi.NO_PATTERN, _abi.BAD_PATTERN) or (
                raise_on_status and st):
            self._check(st, "solve_transpose_device")
        return r.as_dict()

    def pattern_outer_device(self, u, v, out, alpha=-1.0):
        """out[k] = alpha * u[i] * v[j] on the pattern (dL/dA = -lam_i x_j)."""
        self._follow_torch()
        self._check(self._L.ocsl_pattern_outer_device(self._h, float(alpha), _dptr(u), _dptr(v),
                                                      _dptr(out)), "pattern_outer")

    def solve_multi_device(self, method, value, B, X, **opts):
        """Several right-hand sides sharing the matrix: B, X are [nrhs, n] CUDA
        tensors; the factor is built once.  Returns a list of result dicts."""
        self._follow_torch()
        nrhs = int(B.shape[0])
        o = _abi.default_opts(**opts)
        res = (Result * nrhs)()
        st = self._L.ocsl_solve_multi_device(self._h, _method(method), _dptr(value), nrhs,
                                             _dptr(B), _dptr(X), C.byref(o), res)
        if st in (_abi.CUDA_ERROR, _abi.BAD_ARGUMENT, _abi.NO_PATTERN):
            self._check(st, "solve_multi_device")
        return [r.as_dict() for r in res]

    # -- triangular-sweep kernel choice
    def set_sweep_kernel(self, kind: int = 0, tile_a: int = 0, tile_b: int = 0):
        """0 automatic, 1 level-scheduled, 2 structured CTA kernel (tile_a x
        tile_b column tile), 3 structured warp-pipelined kernel (tile_a warps
        per CTA, tile_b start lag); 2 and 3 need a 7-point box pattern."""
        self._check(self._L.ocsl_set_sweep_kernel(self._h, kind, tile_a, tile_b), "sweep kernel")

    def set_sweep_cluster(self, cx: int = 1, cy: int = 1):
        """Run the structured sweep's column tiles in thread-block clusters of
        cx x cy tiles (faces through distributed shared memory); 1 x 1 = none,
        0 x 0 = automatic (the default: 2 x 4 on a grid of at least 64 tiles)."""
        self._check(self._L.ocsl_set_sweep_cluster(self._h, cx, cy), "sweep cluster")

    def sweep_info(self):
        kind = C.c_int()
        dims = (C.c_int * 3)()
        tiles = (C.c_int * 2)()
        self._check(self._L.ocsl_sweep_info(self._h, C.byref(kind), dims, tiles), "sweep_info")
        out = {"kind": kind.value, "dims": tuple(dims)}
        for fp32, suffix in ((0, ""), (1, "32")):
            t, cl = (C.c_int * 2)(), (C.c_int * 2)()
            self._check(self._L.ocsl_sweep_geometry(self._h, fp32, t, cl), "sweep_geometry")
            out["tiles" + suffix] = tuple(t)
            out["cluster" + suffix] = tuple(cl)
            on, wa, lag = C.c_int(), C.c_int(), C.c_int()
            self._check(self._L.ocsl_wave_geometry(self._h, fp32, C.byref(on), C.byref(wa),
                                                   C.byref(lag)), "wave_geometry")
            out["wave" + suffix] = {"on": bool(on.value), "warps": wa.value, "lag": lag.value}
        return out

    def autotune(self, method, value):
        """Pick the structured sweep's column tile for this matrix by timing the
        candidates (value: CUDA tensor of A); returns {"tiles": (TA, TB),
        "sweep_us": t}, tiles (0, 0) when nothing applies."""
        self._follow_torch()
        ta, tb, us = C.c_int(), C.c_int(), C.c_double()
        self._check(self._L.ocsl_autotune_device(self._h, _method(method), _dptr(value),
                                                 C.byref(ta), C.byref(tb), C.byref(us)),
                    "autotune")
        fp32 = _method(method) == ILU_BICGSTAB_IR32
        info = self.sweep_info()
        return {"tiles": (ta.value, tb.value), "sweep_us": us.value,
                "cluster": info["cluster32" if fp32 else "cluster"],
                "wave": info["wave32" if fp32 else "wave"]}

    def autotune_spmv(self, method, value):
        """Pick the CSR SpMV's lanes per row (1, 4 or 16) for this matrix by
        timing them (value: CUDA tensor of A); returns {"lanes", "spmv_us"}."""
        self._follow_torch()
        lanes, us = C.c_int(), C.c_double()
        self._check(self._L.ocsl_autotune_spmv_device(self._h, _method(method), _dptr(value),
                                                      C.byref(lanes), C.byref(us)),
                    "autotune_spmv")
        return {"lanes": lanes.value, "spmv_us": us.value}

    def set_device_loop(self, enable: bool = True):
        """Run FP32-refined solves with their loops on the device (one graph
        launch per solve, conditional WHILE nodes); results are identical."""
        self._check(self._L.ocsl_set_device_loop(self._h, int(bool(enable))), "set_device_loop")

    def set_spmv_lanes(self, lanes: int):
        """CSR SpMV lanes per row: 1 (default), 4 or 16; results are identical."""
        self._check(self._L.ocsl_set_spmv_lanes(self._h, int(lanes)), "set_spmv_lanes")

    def spmv_lanes(self) -> int:
        v = C.c_int()
        self._check(self._L.ocsl_spmv_lanes(self._h, C.byref(v)), "spmv_lanes")
        return v.value

    def set_graphs(self, enable: bool = True):
        """Replay iteration batches from CUDA graphs (default on)."""
        self._check(self._L.ocsl_set_graphs(self._h, int(bool(enable))), "set_graphs")

    def inject_fault(self, kind: int = 1):
        """Test hook: the next triangular sweep leaves out the first unit of its
        schedule, so its bounded waits run out (the call reports OCSL_TIMEOUT);
        kind 0 cancels a pending injection."""
        self._check(self._L.ocsl_inject_fault(self._h, int(kind)), "inject_fault")

    def set_col_batching(self, enable=True):
        """Solve the right-hand sides of solve_multi_device with the FP32-inner
        solver in lockstep groups of up to four (default on).  2: lockstep with
        the SpMM-style box SpMV (each stencil record read once for all
        columns)."""
        mode = enable if isinstance(enable, int) and not isinstance(enable, bool) \
            else int(bool(enable))
        self._check(self._L.ocsl_set_col_batching(self._h, mode), "set_col_batching")

    def set_ordering(self, ordering):
        """Row ordering of the tolerance-mode solves: "natural" (default) or
        "multicolour" (greedy colouring, colour-major renumbering; the solve
        runs on P A P^T and scatters x back)."""
        codes = {"natural": _abi.ORDER_NATURAL, "multicolour": _abi.ORDER_MULTICOLOUR}
        code = codes.get(ordering, ordering)
        self._check(self._L.ocsl_set_ordering(self._h, int(code)), "set_ordering")

    def ordering_info(self):
        """{"ordering", "colours", "levels": (forward, backward), "stencil"}
        of the permuted pattern (zeros until a solve or ordering_permutation
        built it); stencil: red-black box records in use."""
        o, k, st = C.c_int(), C.c_int(), C.c_int()
        lv = (C.c_int32 * 2)()
        self._check(self._L.ocsl_ordering_info(self._h, C.byref(o), C.byref(k), lv,
                                               C.byref(st)), "ordering_info")
        return {"ordering": "multicolour" if o.value == _abi.ORDER_MULTICOLOUR else "natural",
                "colours": k.value, "levels": (lv[0], lv[1]), "stencil": bool(st.value)}

    def ordering_permutation(self):
        """perm[new row] = original row of the multicolour ordering (int32 numpy)."""
        n = self.pattern_info()["n"]
        perm = np.zeros(n, dtype=np.int32)
        self._check(self._L.ocsl_ordering_permutation(
            self._h, perm.ctypes.data_as(C.POINTER(C.c_int32)), n), "ordering_permutation")
        return perm

    # -- kernel timing (ocsl_profile_*)
    def profile(self, enable: bool = True):
        self._check(self._L.ocsl_profile_enable(self._h, int(bool(enable))), "profile_enable")

    def profile_read(self):
        """Per-category device milliseconds and launch counts since the last read."""
        K = _abi.PROFILE_CATEGORIES
        ms = (C.c_double * K)()
        cnt = (C.c_int64 * K)()
        self._check(self._L.ocsl_profile_read(self._h, ms, cnt), "profile_read")
        return {self._L.ocsl_profile_category_name(k).decode(): (ms[k], cnt[k])
                for k in range(K)}

    # -- kernel-level entry points (device tensors)
    def gemv_device(self, value, x, y, mode=0, a=0.0, z=None):
        self._follow_torch()
        self._check(self._L.ocsl_gemv_device(self._h, mode, a, _dptr(value), _dptr(x), _dptr(z),
                                             _dptr(y)), "gemv")

    def dot_device(self, x, y):
        self._follow_torch()
        out = C.c_double()
        self._check(self._L.ocsl_dot_device(self._h, x.numel(), _dptr(x), _dptr(y),
                                            C.byref(out)), "dot")
        return out.value

    def sum_device(self, x, absolute=False):
        """cmatrix_solver.cpp:244-263 sum / ABSsum (tile order)."""
        self._follow_torch()
        out = C.c_double()
        self._check(self._L.ocsl_sum_device(self._h, x.numel(), _dptr(x), int(bool(absolute)),
                                            C.byref(out)), "sum")
        return out.value

    def product_device(self, x, y, out):
        self._follow_torch()
        self._check(self._L.ocsl_product_device(self._h, x.numel(), _dptr(x), _dptr(y),
                                                _dptr(out)), "product")

    def axpy_device(self, a, x, out, b=0.0, y=None):
        """out = a x + b y (the reference's axpy, :275-335); y None: out = a x."""
        self._follow_torch()
        self._check(self._L.ocsl_axpy_device(self._h, x.numel(), float(a), _dptr(x), float(b),
                                             _dptr(y), _dptr(out)), "axpy")

    def ilu_device(self, A, M, sweeps=3):
        self._follow_torch()
        self._check(self._L.ocsl_ilu_device(self._h, _dptr(A), _dptr(M), sweeps), "ilu")

    def forsub_device(self, M, b, y):
        self._follow_torch()
        self._check(self._L.ocsl_forsub_device(self._h, _dptr(M), _dptr(b), _dptr(y)), "forsub")

    def backsub_device(self, M, y, x):
        self._follow_torch()
        self._check(self._L.ocsl_backsub_device(self._h, _dptr(M), _dptr(y), _dptr(x)),
                    "backsub")


def build_pattern(n, left, right, bc_left):
    """The reference's CSR pattern (row_ptr, column_index as uint64, phantom
    2**64-1 on boundary cells) from face connectivity, in O(n + faces)
    (ocsl_build_pattern; replaces cfvm.cpp:74-98).  Host only."""
    L = _abi.lib()
    l = np.ascontiguousarray(left, dtype=np.int32)
    r = np.ascontiguousarray(right, dtype=np.int32)
    b = np.ascontiguousarray(bc_left, dtype=np.int32)
    nnz = C.c_size_t(0)
    st = L.ocsl_build_pattern(int(n), l.size, _ptr(l), _ptr(r), b.size, _ptr(b), None, None,
                              C.byref(nnz))
    if st != 0:
        raise OcslError(st, "build_pattern: bad face connectivity")
    rp = np.zeros(int(n) + 1, dtype=np.uint64)
    col = np.zeros(nnz.value, dtype=np.uint64)
    st = L.ocsl_build_pattern(int(n), l.size, _ptr(l), _ptr(r), b.size, _ptr(b), _ptr(rp),
                              _ptr(col), C.byref(nnz))
    if st != 0:
        raise OcslError(st, "build_pattern")
    return rp, col


class Batch:
    """Many independent systems solved concurrently (ocsl_batch_*): one
    context per system, ``workers`` host threads each driving its own stream.
    ``systems`` is a list of (row_ptr, column_index, nrhs)."""

    def __init__(self, systems, device: int = 0, workers: int = 8):
        self._L = _abi.lib()
        self._keep = []
        arr = (_abi.BatchSystem * len(systems))()
        self.nrhs = []
        self.n = []
        for i, (rp, col, nrhs) in enumerate(systems):
            rp, col = _u64(rp), _u64(col)
            self._keep += [rp, col]
            arr[i].n, arr[i].nrhs = rp.size - 1, int(nrhs)
            arr[i].row_ptr, arr[i].column_index = rp.ctypes.data, col.ctypes.data
            self.nrhs.append(int(nrhs))
            self.n.append(rp.size - 1)
        h = C.c_void_p()
        st = self._L.ocsl_batch_create(C.byref(h), int(device), len(systems), arr, int(workers))
        if st != 0:
            raise OcslError(st, f"batch_create: {self._L.ocsl_status_string(st).decode()}: "
                                f"{self._L.ocsl_last_error(None).decode()}")
        self._h = h
        self._keep = []

    def close(self):
        if getattr(self, "_h", None):
            self._L.ocsl_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_graph(self, enable: bool = True):
        """One graph launch for every FP32-refined solve of the batch, all loops
        on the device (ocsl_batch_set_graph); results are identical."""
        st = self._L.ocsl_batch_set_graph(self._h, int(bool(enable)))
        if st:
            raise OcslError(st, "batch_set_graph")

    def solve_device(self, method, values, Bs, Xs, **opts):
        """values[i], Bs[i] ([nrhs_i, n_i]) and Xs[i] are CUDA tensors; returns
        (status, list of per-right-hand-side result dicts).  The batch's workers
        run on their own streams: pending torch work is finished first."""
        import torch

        torch.cuda.synchronize()
        k = len(values)
        P = C.c_void_p * k
        pv = P(*[_dptr(t).value for t in values])
        pb = P(*[_dptr(t).value for t in Bs])
        px = P(*[_dptr(t).value for t in Xs])
        o = _abi.default_opts(**opts)
        res = (Result * sum(self.nrhs))()
        st = self._L.ocsl_batch_solve_device(self._h, _method(method), pv, pb, px, C.byref(o), res)
        if st in (_abi.CUDA_ERROR, _abi.BAD_ARGUMENT):
            raise OcslError(st, self._L.ocsl_batch_last_error(self._h).decode())
        return st, [r.as_dict() for r in res]


class CMatrix_solver:
    """Mirror of the reference class (cmatrix_solver.h:27-95) on the GPU library.

    Members keep the reference's names and layout; ``CG_solve`` and
    ``ILU_BICGSTAB_solve`` return what the reference returns (absolute /
    relative squared residual) and overwrite ``x_vector.value``.  The pattern is
    uploaded on the first solve and again only if row_ptr / column_index change.
    """

    class CCSR:
        def __init__(self, n_rows=0, n_columns=0, n_nnz=0):
            self.n_rows, self.n_columns, self.n_nnz = n_rows, n_columns, n_nnz
            self.value = np.zeros(0)
            self.row_ptr = np.zeros(n_rows + 1, np.uint64)
            self.column_index = np.zeros(0, np.uint64)

        def clear(self):  # cmatrix_solver.cpp:154-175
            self.value[:] = 0.0

    class Cvector:
        def __init__(self, n_values=0):
            self.n_values = n_values
            self.value = np.zeros(n_values)

        def clear(self):  # cmatrix_solver.cpp:209-230
            self.value[:] = 0.0

    def __init__(self, n_rows=0, n_columns=0, n_nnz=0, device=0, method="bicgstab_ref"):
        self.matrix = self.CCSR(n_rows, n_columns, n_nnz)
        self.b_vector = self.Cvector(n_rows)
        self.x_vector = self.Cvector(n_rows)
        self.method = method  # the reference's global MATRIX_SOLVER_TYPE
        self.last_result = None
        self._ctx = Context(device)
        self._pattern_key = None

    def _sync_pattern(self):
        rp, col = _u64(self.matrix.row_ptr), _u64(self.matrix.column_index)
        key = (rp.size, col.size, hash(rp.tobytes()), hash(col.tobytes()))
        if key != self._pattern_key:
            self._ctx.set_pattern(rp, col)
            self._pattern_key = key

    def _run(self, method, **opts):
        self._sync_pattern()
        x = np.ascontiguousarray(self.x_vector.value, dtype=np.float64).copy()
        r = self._ctx.solve(method, self.matrix.value, self.b_vector.value, x, **opts)
        if r["status"] not in (0, _abi.NOT_CONVERGED):
            raise OcslError(r["status"], f"solve: {_abi.status_string(r['status'])}")
        self.x_vector.value = x
        self.last_result = r
        return r

    def CG_solve(self):
        """cmatrix_solver.cpp:635-680: 4 iterations, returns ||r||^2."""
        return self._run(CG_REF)["residual"]

    def ILU_BICGSTAB_solve(self):
        """cmatrix_solver.cpp:682-762: ILU + 3 iterations, returns ||r||^2/||b||^2."""
        return self._run(BICGSTAB_REF)["residual"]

    def solve(self, method=None, **opts):
        """cmatrix_solver.cpp:764-780, with the method chosen per call."""
        return self._run(_method(method if method is not None else self.method), **opts)


def read_su2(path: str) -> dict:
    """Read an SU2 ASCII mesh into the finite-volume arrays of ocsl_mesh_arrays
    (numpy copies, vectors [3][count]) plus "markers" (names, in file order),
    with the reference's face numbering (ocsl_mesh_read_su2)."""
    L = _abi.lib()
    h = C.c_void_p()
    err = C.create_string_buffer(512)
    st = L.ocsl_mesh_read_su2(os.fsencode(path), C.byref(h), err, 512)
    if st != 0:
        raise OcslError(st, f"read_su2: {err.value.decode()}")
    try:
        v = _abi.MeshArrays()
        L.ocsl_mesh_view(h, C.byref(v))
        out = {"n_cells": v.n_cells, "n_faces": v.n_faces, "n_bc": v.n_bc}
        for name, kind, comps, count in _abi.MESH_ARRAYS:
            size = comps * int(getattr(v, count))
            ptr = getattr(v, name)
            dt = np.int32 if kind == "i" else np.float64
            out[name] = np.ctypeslib.as_array(ptr, shape=(size,)).astype(dt, copy=True) \
                if size else np.zeros(0, dt)
        out["markers"] = [L.ocsl_mesh_marker_name(h, k).decode() for k in range(v.n_markers)]
        return out
    finally:
        L.ocsl_mesh_destroy(h)


class Mesh:
    """An SU2 mesh held by the library (ocsl_mesh_read_su2) for VTK output of a
    solution on it (ocsl_vtk_write), as Cpost_processing writes it."""

    def __init__(self, path: str):
        self._L = _abi.lib()
        self._h = C.c_void_p()
        err = C.create_string_buffer(512)
        st = self._L.ocsl_mesh_read_su2(os.fsencode(path), C.byref(self._h), err, 512)
        if st != 0:
            raise OcslError(st, f"read_su2: {err.value.decode()}")
        v = _abi.MeshArrays()
        self._L.ocsl_mesh_view(self._h, C.byref(v))
        self.n_cells, self.n_faces, self.n_bc = int(v.n_cells), int(v.n_faces), int(v.n_bc)

    def close(self) -> None:
        if self._h:
            self._L.ocsl_mesh_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _field(a, keep: list, dtype):
        """Pointer to a field: a CUDA tensor stays on the device (the writer
        streams it), anything else is made a contiguous host array."""
        if a is None:
            return None
        if hasattr(a, "is_cuda") and a.is_cuda:
            keep.append(a)
            return a.data_ptr()
        h = np.ascontiguousarray(a.cpu().numpy() if hasattr(a, "cpu") else a, dtype)
        keep.append(h)
        return h.ctypes.data

    def write_vtk(self, cells_path=None, boundary_path=None, *, heat=False, digits=0,
                  density=None, pressure=None, temperature=None, mach=None, velocity=None,
                  pressure_grad=None, bc_temperature=None, bc_type=None, bc_wall=None,
                  viscous=False, sutherland=(0.0, 0.0)) -> None:
        """Write solution.vtk / solution_BC.vtk of the reference's
        post-processing (either path may be None).  Fields are numpy arrays or
        CUDA tensors; vectors [3][count] (flattened or shaped (3, count))."""
        keep: list = []
        f = _abi.VtkFields()
        f.heat, f.digits, f.viscous = int(bool(heat)), int(digits), int(bool(viscous))
        for name, a in (("density", density), ("pressure", pressure),
                        ("temperature", temperature), ("mach", mach), ("velocity", velocity),
                        ("pressure_grad", pressure_grad), ("bc_temperature", bc_temperature)):
            setattr(f, name, self._field(a, keep, np.float64))
        f.bc_type = self._field(bc_type, keep, np.int32)
        f.bc_wall = self._field(bc_wall, keep, np.int32)
        f.sutherland[0], f.sutherland[1] = float(sutherland[0]), float(sutherland[1])
        err = C.create_string_buffer(512)
        enc = (lambda p: None if p is None else os.fsencode(str(p)))  # noqa: E731
        st = self._L.ocsl_vtk_write(self._h, C.byref(f), enc(cells_path), enc(boundary_path),
                                    err, 512)
        if st != 0:
            raise OcslError(st, f"write_vtk: {err.value.decode()}")
