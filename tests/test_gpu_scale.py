"""Parity at full size.

* Face-loop assembly on the 128^3 hex flow state (2,097,152 cells, 6,242,304
  interior faces) and on a tet mesh: the GPU kernel equals the oracle
  restatement bit for bit (values, b, x0, ap, total_mdot) for the pressure
  correction, the three momentum components (inviscid and viscous), the
  enthalpy and the heat-conduction equation.
* Mixed precision: on the hex 128^3 p' system (Peclet <= 10) and the tet
  64^3 x 6 system (Peclet <= 50), the FP32-inner / FP64-refined solve and
  the plain FP64 solve both reach 1e-10; each one's error against the CPU
  oracle's FP64 solution taken to 1e-13 is stated, and the FP32-refined
  error must be within 2x the plain FP64 solve's error.
"""
import os

import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import workloads as W
from oracle import oracle as orc

import assembly_cases as AC

pytestmark = pytest.mark.gpu


def _equations(eq0):
    out = [("pressure", dict(eq0, equation=_abi.EQ_PRESSURE, dimension=0))]
    for d in range(3):
        for visc in (0, 1):
            out.append((f"momentum_{'xyz'[d]}_visc{visc}",
                        dict(eq0, equation=_abi.EQ_MOMENTUM, dimension=d, viscous=visc)))
    out.append(("enthalpy", dict(eq0, equation=_abi.EQ_ENTHALPY, dimension=0, viscous=1)))
    out.append(("heat", {"equation": _abi.EQ_HEAT, "transient": 1, "thermal_diffusivity": 2.2e-5}))
    return out


def _check_assembly(ctx, torch, f):
    ctx.set_pattern(f.row_ptr, f.column_index)
    ctx.set_faces(f.left, f.right, f.bc_left)
    st = AC.to_device(torch, f.state)
    n, nnz = f.n, f.column_index.size
    value = torch.empty(nnz, dtype=torch.float64, device="cuda")
    b, x0, ap, tm = (torch.empty(n, dtype=torch.float64, device="cuda") for _ in range(4))
    for name, eq in _equations(f.eq):
        for t in (value, b, x0, ap, tm):
            t.fill_(float("nan"))
        ctx.assemble_device(eq, st, value, b, x0, ap, tm)
        got = [t.cpu().numpy() for t in (value, b, x0, ap, tm)]
        want = orc.assemble(f.row_ptr, f.column_index, f.left, f.right, f.bc_left, eq, f.state)
        for g, w, what in zip(got, want, ("value", "b", "x0", "ap", "total_mdot")):
            if name == "heat" and what in ("ap", "total_mdot"):
                continue  # the heat solver has neither (cheat_solver.cpp:57-65)
            assert np.array_equal(g, w), (f.name, name, what)
        assert np.all(np.isfinite(got[0])) and np.all(np.isfinite(got[1])), (f.name, name)


def _with_viscous_state(f, seed):
    st = dict(f.state)
    rng = np.random.default_rng(seed)
    st["stress"] = rng.uniform(-1.0, 1.0, (3, f.left.size)) * 1e-3
    st["bc_thermal"] = (np.arange(f.bc_left.size) % 2).astype(np.int32)
    st["pressure_grad"] = rng.uniform(-1.0, 1.0, (3, f.n))
    st["pressure_corr"] = rng.uniform(-1.0, 1.0, f.n)
    f.state = st
    return f


def test_assembly_hex128_bit_exact(ctx, torch_cuda):
    f = _with_viscous_state(W.hex_flow_state(128), 5)
    _check_assembly(ctx, torch_cuda, f)


def test_assembly_tet_bit_exact(ctx, torch_cuda):
    _check_assembly(ctx, torch_cuda, W.tet_flow_state(20))


@pytest.fixture(scope="module")
def cpu_oracle():
    o = orc.Oracle()
    o.set_threads(os.cpu_count() or 1)
    return o


def _err(x, xr):
    return float(np.linalg.norm(x - xr) / np.linalg.norm(xr))


@pytest.mark.parametrize("which", ["hex128", "tet64"])
def test_fp32_refined_error_vs_fp64_oracle(ctx, cpu_oracle, hex128, which):
    s = hex128 if which == "hex128" else W.tet_pprime(64, peclet=50.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    x0 = np.zeros(s.n)
    x_ref, rc, it_ref, _ = cpu_oracle.bicgstab_tol(s.row_ptr, s.column_index, s.value, s.b, x0,
                                                   tol=1e-13, maxit=4000)
    assert rc == 0, (rc, it_ref)
    assert cpu_oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x_ref) <= 1e-13
    res = {}
    for name, method in (("fp64", ocsl.ILU_BICGSTAB), ("fp32_refined", ocsl.ILU_BICGSTAB_IR32)):
        x = x0.copy()
        r = ctx.solve(method, s.value, s.b, x, tol=1e-10)
        assert r["status"] == 0, (name, r)
        rr = cpu_oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x)
        assert rr <= 1e-10, (name, rr)
        res[name] = _err(x, x_ref)
    print(f"{which}: error vs FP64 oracle (1e-13): fp64 {res['fp64']:.3e}, "
          f"fp32_refined {res['fp32_refined']:.3e}")
    assert res["fp32_refined"] <= 2.0 * res["fp64"], res
