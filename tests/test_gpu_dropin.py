"""The C++ drop-in over the real library, as one program: C++17 host code
calling CMatrix_solver::solve() / CG_solve() / ILU_BICGSTAB_solve() on one
solver object, linked with -Wl,--wrap into the drop-in
(opencslsolver_gb300/shim/cmatrix_solver_gpu.cpp), which calls
libocsl_gb300.so through the C ABI.

The host program (tests/shim_host/replay.cpp) replays the solve calls recorded
from the reference's own SIMPLE loop on the 1000-cell shock tube with the
per-equation dispatch of that case (momentum through CG, pressure correction
and enthalpy through ILU-BiCGSTAB).  The reference's headers are not on the
GPU host, so the drop-in is compiled against a stand-in that declares the
members it uses under the reference's names (tests/shim_host/croot.h).

* On a GPU: every x equals the oracle's bit for bit and the reference's
  recorded x within 1e-12; the direct CG_solve() / ILU_BICGSTAB_solve() calls
  return the reference's residuals; solve() accounts its time into
  root.total_elapsed_matrix_solution_time; OCSL_SOLVER selects a tolerance-mode
  method.
* Without a GPU (CPU suite): the program stops with the library's error
  instead of falling back to a CPU solve.
"""
import os
import subprocess

import numpy as np
import pytest

from opencslsolver_gb300 import _abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HOST = os.path.join(ROOT, "tests", "shim_host")
SHIM = os.path.join(ROOT, "opencslsolver_gb300", "shim", "cmatrix_solver_gpu.cpp")
WRAP = ["-Wl,--wrap=_ZN14CMatrix_solver5solveEv", "-Wl,--wrap=_ZN14CMatrix_solver8CG_solveEv",
        "-Wl,--wrap=_ZN14CMatrix_solver18ILU_BICGSTAB_solveEv"]


def build_replay(out_dir):
    lib_dir = os.path.dirname(_abi.LIB_PATH)
    exe = os.path.join(str(out_dir), "replay")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-I", HOST, "-I",
           os.path.join(ROOT, "include"), SHIM, os.path.join(HOST, "replay.cpp"), *WRAP,
           "-L", lib_dir, "-locsl_gb300", f"-Wl,-rpath,{lib_dir}", "-o", exe]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def write_calls(path, rp, col, calls):
    n, nnz = rp.size - 1, col.size
    with open(path, "wb") as f:
        np.array([n, nnz, len(calls)], np.uint64).tofile(f)
        rp.astype(np.uint64).tofile(f)
        col.astype(np.uint64).tofile(f)
        for method, val, b, x0 in calls:
            np.array([method], np.int32).tofile(f)
            np.ascontiguousarray(val, np.float64).tofile(f)
            np.ascontiguousarray(b, np.float64).tofile(f)
            np.ascontiguousarray(x0, np.float64).tofile(f)


def read_out(path, n, ncalls):
    raw = np.fromfile(path, np.uint8)
    body = raw[:ncalls * (n + 1) * 8].view(np.float64).reshape(ncalls, n + 1)
    us = int(raw[ncalls * (n + 1) * 8:].view(np.uint64)[0])
    return body[:, :n], body[:, n], us


def shocktube_calls(z):
    calls = []
    for k in range(z["meta"].shape[0]):
        eq = int(z["meta"][k, 2])
        calls.append((0 if eq < 3 else 1, z["value"][k], z["b"][k], z["x0"][k]))
    return calls


def test_dropin_builds_and_refuses_without_gpu(lib_built, golden_shocktube, tmp_path):
    import torch

    exe = build_replay(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("host has a GPU (covered by the GPU test)")
    z = golden_shocktube
    write_calls(tmp_path / "calls.bin", z["row_ptr"], z["column_index"], shocktube_calls(z)[:1])
    p = subprocess.run([exe, str(tmp_path / "calls.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=120)
    assert p.returncode == 1
    assert "ocsl: ocsl_create failed" in p.stderr


@pytest.mark.gpu
def test_dropin_replays_shocktube_calls_on_gpu(lib_built, torch_cuda, oracle, golden_shocktube,
                                               golden_kat, tmp_path):
    z = golden_shocktube
    rp, col = z["row_ptr"], z["column_index"]
    calls = shocktube_calls(z)
    # the reference's solver unit-test system, called directly (cmatrix_solver_supply.h:78,110)
    k = golden_kat
    exe = build_replay(tmp_path)
    write_calls(tmp_path / "calls.bin", rp, col, calls)
    p = subprocess.run([exe, str(tmp_path / "calls.bin"), str(tmp_path / "out.bin")],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    xs, res, us = read_out(tmp_path / "out.bin", rp.size - 1, len(calls))
    for i, (method, val, b, x0) in enumerate(calls):
        fn = oracle.cg_ref if method == 0 else oracle.bicgstab_ref
        xo, _, _ = fn(rp, col, val, b, x0)
        assert np.array_equal(xs[i], xo), i
        scale = max(float(np.max(np.abs(z["x"][i]))), 1e-300)
        assert float(np.max(np.abs(xs[i] - z["x"][i]))) / scale <= 1e-12, i
    assert us > 0  # solve() added its elapsed time, as cmatrix_solver.cpp:779 does
    print(f"{len(calls)} solve() calls through the drop-in: {us / len(calls):.0f} us per call")

    kcalls = [(2, k["value"], k["b"], k["x0"]), (3, k["value"], k["b"], k["x0"])]
    write_calls(tmp_path / "kat.bin", k["row_ptr"], k["column_index"], kcalls)
    p = subprocess.run([exe, str(tmp_path / "kat.bin"), str(tmp_path / "kat.out")],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    kx, kres, _ = read_out(tmp_path / "kat.out", 10, 2)
    np.testing.assert_allclose(kres[0], float(k["cg_res"]), rtol=1e-12)
    np.testing.assert_allclose(kres[1], float(k["bicg_res"]), rtol=1e-9)
    np.testing.assert_allclose(kx[0], k["cg_x"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(kx[1], k["bicg_x"], rtol=0, atol=1e-14)

    # OCSL_SOLVER: solve() runs a tolerance-mode method instead
    pcalls = [c for c in calls if c[0] == 1][:2]
    write_calls(tmp_path / "tol.bin", rp, col, pcalls)
    env = dict(os.environ, OCSL_SOLVER="ilu_bicgstab_ir32", OCSL_TOL="1e-11")
    p = subprocess.run([exe, str(tmp_path / "tol.bin"), str(tmp_path / "tol.out")],
                       capture_output=True, text=True, timeout=300, env=env)
    assert p.returncode == 0, p.stderr
    tx, _, _ = read_out(tmp_path / "tol.out", rp.size - 1, len(pcalls))
    for i, (_, val, b, _) in enumerate(pcalls):
        assert oracle.true_relres(rp, col, val, b, tx[i]) <= 1e-11


# ---------------------------------------------------------------------------
# The shock tube's whole SIMPLE loop with every solve through the drop-in.
# The host-side stages of CFlow_solver::iterate (boundary conditions,
# gradients, assembly, mass fluxes, corrections, field updates) are the
# oracle's restatement (oracle/ocsl_oracle_flow.c), standing in for the
# reference's own flow solver, which cannot be built where the GPU is; each of
# the five solves of an inner iteration goes through CMatrix_solver::solve()
# of one solver object (tests/shim_host/simple_host.cpp) into the C++ drop-in
# and libocsl_gb300.so, with the dispatch of the 1000-cell case: momentum CG,
# pressure correction and enthalpy ILU-BiCGSTAB, 200 steps x 5 inner
# iterations, pattern uploaded once.

CG_METHODS = (0, 1, 1)  # OCSL_CG_REF for momentum, OCSL_BICGSTAB_REF for p' and enthalpy


def build_simple_host(out_dir):
    lib_dir = os.path.dirname(_abi.LIB_PATH)
    so = os.path.join(str(out_dir), "libsimple_host.so")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-Wextra", "-fPIC", "-shared", "-I", HOST,
           "-I", os.path.join(ROOT, "include"), SHIM, os.path.join(HOST, "simple_host.cpp"),
           *WRAP, "-L", lib_dir, "-locsl_gb300", f"-Wl,-rpath,{lib_dir}", "-o", so]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return so


def _simple_loop(solve_with, steps=None):
    """Runs the shock tube from its recorded set-up; ``solve_with`` None uses
    the oracle's own reference-faithful solves, else a path to the built
    simple_host library.  Returns the written fields and the loop's time."""
    import ctypes
    import sys
    import time

    sys.path.insert(0, HERE_TESTS)
    import flow_cases as FC
    from oracle import oracle as orc

    g = FC.Golden("shocktube")
    c = g.case()
    fn = lib = None
    if solve_with:
        lib = ctypes.CDLL(solve_with)
        lib.simple_host_set_pattern.argtypes = [ctypes.c_size_t, ctypes.c_void_p,
                                                ctypes.c_void_p]
        lib.simple_host_elapsed_us.restype = ctypes.c_ulonglong
        rp = np.ascontiguousarray(c["row_ptr"], np.uint64)
        col = np.ascontiguousarray(c["column_index"], np.uint64)
        lib.simple_host_set_pattern(rp.size - 1, rp.ctypes.data, col.ctypes.data)
        fn = lib.simple_host_solve
    t0 = time.perf_counter()
    for _ in range(steps or g.steps):
        for _ in range(g.inner):
            if fn is not None:
                orc.flow_iterate_with(c, CG_METHODS, fn)
            else:
                orc.flow_iterate(c, CG_METHODS)
        FC.end_step(c, orc.flow_end_step)
    wall = time.perf_counter() - t0
    out = {k: np.array(v) for k, v in FC.written(c).items()}
    out["_wall_s"] = np.array(wall)
    out["_solve_us"] = np.array(lib.simple_host_elapsed_us() if lib else 0)
    out["_inner"] = np.array((steps or g.steps) * g.inner)
    return out


HERE_TESTS = os.path.join(ROOT, "tests")


def test_simple_host_builds_and_refuses_without_gpu(lib_built, tmp_path):
    import sys

    import torch

    so = build_simple_host(tmp_path)
    if torch.cuda.is_available():
        pytest.skip("host has a GPU (covered by the GPU test)")
    p = subprocess.run([sys.executable, os.path.abspath(__file__), "simple-loop", so,
                        str(tmp_path / "out.npz")], capture_output=True, text=True, timeout=300,
                       cwd=ROOT, env=dict(os.environ,
                                          PYTHONPATH=os.pathsep.join([ROOT, HERE_TESTS])))
    assert p.returncode == 1
    assert "ocsl: ocsl_create failed" in p.stderr


@pytest.mark.gpu
def test_dropin_runs_shocktube_simple_loop_on_gpu(lib_built, torch_cuda, oracle, tmp_path):
    import sys

    import flow_cases as FC

    so = build_simple_host(tmp_path)
    out = tmp_path / "gpu_loop.npz"
    # a child process: the drop-in ends its program on a library failure, as
    # the reference ends on its own errors
    p = subprocess.run([sys.executable, os.path.abspath(__file__), "simple-loop", so, str(out)],
                       capture_output=True, text=True, timeout=900, cwd=ROOT,
                       env=dict(os.environ, PYTHONPATH=os.pathsep.join([ROOT, HERE_TESTS])))
    assert p.returncode == 0, p.stderr[-2000:]
    got = dict(np.load(out))
    wall, solve_us, inner = (float(got.pop(k)) for k in ("_wall_s", "_solve_us", "_inner"))
    # the same loop with the oracle's own solves: identical bits, since every
    # drop-in solve equals the oracle's reference-faithful solve bit for bit
    want = _simple_loop(None)
    for k in ("_wall_s", "_solve_us", "_inner"):
        want.pop(k)
    for k in want:
        assert np.array_equal(got[k], want[k]), (k, FC.relerr(got[k], want[k]))
    # and the reference's own run (its final state with momentum through CG)
    g = FC.Golden("shocktube")
    errs = FC.field_errors(got, FC.recorded(g.setup, g.record("final_cg")))
    state = max(errs[k] for k in ("velocity", "pressure", "temperature", "density_c",
                                  "enthalpy", "mdot", "density"))
    print(f"shock tube through the C++ drop-in: {inner:.0f} inner iterations, "
          f"{wall * 1e3 / inner:.2f} ms each ({solve_us / 1e3 / inner:.2f} ms in solve()); "
          f"vs the reference's run: state {state:.2e}, all fields {max(errs.values()):.2e}")
    assert state <= 1e-11, errs
    assert max(errs.values()) <= 1e-8, errs


if __name__ == "__main__":
    import sys

    if len(sys.argv) == 4 and sys.argv[1] == "simple-loop":
        res = _simple_loop(sys.argv[2])
        np.savez(sys.argv[3], **res)
