"""Failure statuses of the GPU path, made from data or on the host -- no GPU
fault, trap or unbounded wait is involved.

* OCSL_ZERO_PIVOT: a matrix whose factor has a zero diagonal.  The
  reference-faithful method still computes what the reference computes (its
  pivot check is commented out, cmatrix_solver.cpp:495-500) and reports the
  status -- every entry that stays finite equals the oracle's; where
  infinities appear, the reference also multiplies them by the zeros of
  absent pattern entries (NaN), which the product table leaves out, so only
  the finite entries are compared; tolerance-mode methods run no iteration
  and leave x unchanged.
* OCSL_TIMEOUT: ocsl_inject_fault makes the next triangular sweep leave out the
  first tile / chunk of its schedule, so the waits on those rows run out after
  their bound.  The call must return OCSL_TIMEOUT, and the same context must
  then solve bit-identically to the oracle.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import _abi
from opencslsolver_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _zero_first_pivot(s):
    """Row 0 has no lower entries, so M_00 = A_00 after every fixed-point sweep:
    A_00 = 0 makes the factor's first pivot zero."""
    v = s.value.copy()
    rp = s.row_ptr.astype(np.int64)
    col = s.column_index
    for q in range(rp[0], rp[1]):
        if col[q] == 0:
            v[q] = 0.0
    return W.System(s.row_ptr, s.column_index, v, s.b)


def _same_where_finite(got, want):
    both = np.isfinite(got) & np.isfinite(want)
    np.testing.assert_array_equal(got[both], want[both])


@pytest.mark.parametrize("make", [lambda: W.hex_pprime(10, peclet=10.0),
                                  lambda: W.tet_pprime(4, peclet=50.0)], ids=["hex", "tet"])
def test_zero_pivot(ctx, oracle, make):
    s = _zero_first_pivot(make())
    ctx.set_pattern(s.row_ptr, s.column_index)
    x0 = np.linspace(-1.0, 1.0, s.n)
    # reference-faithful: the oracle's bits wherever both stay finite, status reported
    x = x0.copy()
    r = ctx.solve(ocsl.BICGSTAB_REF, s.value, s.b, x)
    assert r["status"] == _abi.ZERO_PIVOT
    xo, res_o, _ = oracle.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
    _same_where_finite(x, xo)
    assert b"pivot" in ctx._L.ocsl_last_error(ctx._h)
    # tolerance mode: nothing runs, x is left as it was
    for m in (ocsl.ILU_BICGSTAB, ocsl.ILU_BICGSTAB_IR32, ocsl.PCG):
        x = x0.copy()
        r = ctx.solve(m, s.value, s.b, x)
        assert r["status"] == _abi.ZERO_PIVOT, (m, r)
        assert r["iterations"] == 0 and np.array_equal(x, x0)
    # the context is fine with a good matrix afterwards
    g = make()
    x = np.zeros(g.n)
    r = ctx.solve(ocsl.ILU_BICGSTAB, g.value, g.b, x, tol=1e-10)
    assert r["status"] == 0
    assert oracle.true_relres(g.row_ptr, g.column_index, g.value, g.b, x) <= 1e-10


def test_ilu_entry_reports_zero_pivot(ctx, oracle, torch_cuda):
    torch = torch_cuda
    s = _zero_first_pivot(W.hex_pprime(6))
    ctx.set_pattern(s.row_ptr, s.column_index)
    A = torch.from_numpy(s.value).cuda()
    M = torch.zeros_like(A)
    with pytest.raises(ocsl.OcslError) as e:
        ctx.ilu_device(A, M, sweeps=3)
    assert e.value.status == _abi.ZERO_PIVOT
    # M is still written, as the reference's ILU_decompose writes it
    Mo = oracle.ilu(s.row_ptr, s.column_index, s.value, 3)
    m = M.cpu().numpy()
    assert not np.all(np.isfinite(m))
    _same_where_finite(m, Mo)


@pytest.mark.parametrize("case", ["box", "box_clusters", "wave", "level"])
def test_sweep_wait_runs_out(ctx, oracle, case):
    """A sweep whose first tile never runs: its bounded waits give up, the solve
    reports OCSL_TIMEOUT, and the context then solves exactly as before."""
    if case == "level":
        s = W.tet_pprime(5, peclet=50.0)
    else:
        s = W.hex_pprime(24, 70, 20, peclet=10.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    if case == "box":
        ctx.set_sweep_kernel(2, 8, 8)
        ctx.set_sweep_cluster(1, 1)
    elif case == "box_clusters":
        ctx.set_sweep_kernel(2, 8, 4)
        ctx.set_sweep_cluster(2, 2)
    elif case == "wave":
        ctx.set_sweep_kernel(3, 2, 0)  # 3 x 3 CTAs of 2 warps
    kind = {"level": 1, "wave": 3}.get(case, 2)
    assert ctx.sweep_info()["kind"] == kind
    x0 = np.zeros(s.n)
    xo, res_o, it_o = oracle.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, x0)
    for method in (ocsl.BICGSTAB_REF, ocsl.ILU_BICGSTAB_IR32):
        ctx.inject_fault(1)
        x = x0.copy()
        r = ctx.solve(method, s.value, s.b, x, tol=1e-10, maxit=20)
        assert r["status"] == _abi.TIMEOUT, (method, r)
        assert b"bound" in ctx._L.ocsl_last_error(ctx._h)
        # the injection was consumed: the next solve is the oracle's, bit for bit
        x = x0.copy()
        r = ctx.solve(ocsl.BICGSTAB_REF, s.value, s.b, x)
        assert r["status"] == 0
        assert np.array_equal(x, xo) and r["residual"] == res_o and r["iterations"] == it_o


def test_inject_fault_arguments(ctx):
    with pytest.raises(ocsl.OcslError) as e:
        ctx.inject_fault(7)
    assert e.value.status == _abi.BAD_ARGUMENT
    # a cancelled injection changes nothing
    s = W.hex_pprime(8)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.inject_fault(1)
    ctx.inject_fault(0)
    x = np.zeros(s.n)
    assert ctx.solve(ocsl.BICGSTAB_REF, s.value, s.b, x)["status"] == 0
