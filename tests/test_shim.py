"""The C++ drop-in (opencslsolver_gb300/shim/cmatrix_solver_gpu.cpp) linked
into the reference's own, unmodified program with ``--wrap`` (oracle/Makefile
``shim``), on CPU.

* The reference's solver unit tests (cmatrix_solver_supply.h:29-114) call
  CG_solve() / ILU_BICGSTAB_solve() directly; through the drop-in they must
  print the residuals the reference's solver returns (golden KAT).
* The reference's SIMPLE loop on the 1000-cell shock tube calls solve()
  (cflow_solver.cpp:289,349,460); through the drop-in over an oracle-backed
  fake of the C ABI its final fields must equal the run on the reference's own
  solver to round-off, with the pattern uploaded once.
* Over the real GPU library on a host without a GPU the program must stop
  with the library's error, not fall back to a CPU solve.

The drivers link the reference's sources, so these tests run where those are
present and skip elsewhere.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from oracle import oracle as orc

pytestmark = pytest.mark.skipif(not orc.reference_sources_present(),
                                reason="needs the reference's sources to link the drivers")


@pytest.fixture(scope="module")
def drivers(lib_built):
    return orc.build_shim_drivers()


def _run(exe, args, tmp_path, env=None):
    e = dict(os.environ)
    e.update(env or {})
    return subprocess.run([exe] + args, cwd=tmp_path, env=e, capture_output=True, text=True,
                          timeout=300)


def test_unit_tests_route_to_dropin(drivers, tmp_path, golden_kat):
    p = _run(drivers["fake"], ["unit"], tmp_path, {"FAKE_OCSL_LOG": "1"})
    assert p.returncode == 0, p.stderr
    res = [float(m) for m in re.findall(r"residual 0\.323 to : (\S+)", p.stdout)]
    assert len(res) == 2
    np.testing.assert_allclose(res[0], float(golden_kat["cg_res"]), rtol=1e-12)
    np.testing.assert_allclose(res[1], float(golden_kat["bicg_res"]), rtol=1e-9)
    methods = [int(m) for m in re.findall(r"fake_ocsl: solve \d+ method (\d+)", p.stderr)]
    assert methods == [0, 1]  # CG_solve -> OCSL_CG_REF, ILU_BICGSTAB_solve -> OCSL_BICGSTAB_REF


def test_cg_unit_test_matches_reference_solver(drivers, tmp_path):
    # The reference's own ILU unit test dereferences an unset factor and
    # crashes (cmatrix_solver_supply.h:84-114 never calls
    # extract_diag_indexes), so only its CG line runs to completion here.
    ref = _run(drivers["cpu"], ["unit"], tmp_path)
    dropin = _run(drivers["fake"], ["unit"], tmp_path)
    r_ref = float(re.search(r"CG solver residual 0\.323 to : (\S+)", ref.stdout).group(1))
    r_dropin = float(re.search(r"CG solver residual 0\.323 to : (\S+)", dropin.stdout).group(1))
    np.testing.assert_allclose(r_dropin, r_ref, rtol=1e-12)


@pytest.mark.parametrize("threads", [1, 4])
def test_shocktube_through_dropin(drivers, tmp_path, threads):
    steps, inner = 20, 10
    args = lambda name: ["shocktube", str(tmp_path / name), str(threads), str(steps), str(inner)]
    ref = _run(drivers["cpu"], args("ref.txt"), tmp_path)
    assert ref.returncode == 0, ref.stderr[-2000:]
    dropin = _run(drivers["fake"], args("dropin.txt"), tmp_path, {"FAKE_OCSL_LOG": "1"})
    assert dropin.returncode == 0, dropin.stderr[-2000:]
    a = np.loadtxt(tmp_path / "ref.txt")
    b = np.loadtxt(tmp_path / "dropin.txt")
    assert a.shape == b.shape == (1000, 4)
    # p, u, T, rho; scale-relative: the reference's solver sums its dot
    # products in OpenMP order under -ffast-math, the drop-in in tile order.
    err = np.abs(a - b).max(axis=0) / np.abs(a).max(axis=0)
    assert err.max() < 1e-12, err
    solves = re.findall(r"fake_ocsl: solve (\d+) method (\d+) n (\d+) .* uploads (\d+)",
                        dropin.stderr)
    assert len(solves) == steps * inner * 5  # u, v, w, p', h per inner iteration
    assert {m for _, m, _, _ in solves} == {"1"}  # ILU_BICSTAB switch -> Mode R BiCGSTAB
    assert {n for _, _, n, _ in solves} == {"1000"}
    assert solves[-1][3] == "1"  # the fixed pattern is uploaded once


def test_gpu_dropin_fails_loudly_without_device(drivers, tmp_path):
    import torch

    if torch.cuda.is_available():
        pytest.skip("host has a GPU")
    p = _run(drivers["gpu"], ["shocktube", str(tmp_path / "f.txt"), "1", "1", "1"], tmp_path)
    assert p.returncode == 1
    assert "ocsl: ocsl_create failed" in p.stderr
    assert not (tmp_path / "f.txt").exists()
