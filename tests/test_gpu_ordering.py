"""GPU parity of the multicolour ordering (ocsl_set_ordering).

The library's permutation equals the numpy restatement
(tests/ordering_cases.py), and a tolerance-mode solve through the ordering is
bit-identical to the oracle's solve of the permuted system P A P^T, P b,
P x0 (oracle/ocsl_oracle.c, same algorithm, rounding and tile-order
reductions) scattered back -- x and the iteration count.  The FP32-inner
solver reaches the tolerance; the permuted pattern sweeps in one level per
colour; switching back to natural order gives the natural-order results.
"""
import numpy as np
import pytest

import opencslsolver_gb300 as ocsl
from opencslsolver_gb300 import workloads as W

import ordering_cases as OC

pytestmark = pytest.mark.gpu


def systems():
    """Red-black boxes with even nx (stencil records), a box with odd nx
    (red-black through the CSR kernels) and a 4-colour tet mesh."""
    return [W.hex_pprime(16, peclet=10.0), W.hex_pprime(12, 10, 9, peclet=0.0),
            W.tet_pprime(5, peclet=50.0), W.hex_pprime(9, 8, 7, peclet=10.0)]


def oracle_permuted(oracle, fn, s, x0, **kw):
    perm, _ = OC.colour_order(s.row_ptr, s.column_index)
    rp, col, val, b = OC.permuted_system(s, perm)
    xp, rc, it, rr = fn(rp, col, val, b, np.asarray(x0)[perm], **kw)
    x = np.empty_like(xp)
    x[perm] = xp
    return x, rc, it


@pytest.mark.parametrize("k", range(4))
def test_permutation_and_levels(ctx, k):
    s = systems()[k]
    ctx.set_pattern(s.row_ptr, s.column_index)
    assert ctx.ordering_info() == {"ordering": "natural", "colours": 0, "levels": (0, 0),
                                   "stencil": False}
    ctx.set_ordering("multicolour")
    perm = ctx.ordering_permutation()
    want, colours = OC.colour_order(s.row_ptr, s.column_index)
    assert np.array_equal(perm, want)
    info = ctx.ordering_info()
    assert info["ordering"] == "multicolour" and info["colours"] == colours
    assert info["levels"] == (colours, colours)
    if k < 2:  # even-nx boxes: red-black stencil records
        assert colours == 2 and info["stencil"]
    else:
        assert not info["stencil"]


@pytest.mark.parametrize("k", range(4))
def test_multicolour_bicgstab_bit_exact(ctx, oracle, k):
    s = systems()[k]
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_ordering("multicolour")
    for x0 in (np.zeros(s.n), np.random.default_rng(k).uniform(-1, 1, s.n)):
        x = x0.copy()
        r = ctx.solve(ocsl.ILU_BICGSTAB, s.value, s.b, x, tol=1e-10)
        assert r["status"] == 0, r
        xo, rc, it = oracle_permuted(oracle, oracle.bicgstab_tol, s, x0, tol=1e-10)
        assert rc == 0
        assert np.array_equal(x, xo) and r["iterations"] == it
        assert oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x) <= 1e-10


def test_multicolour_pcg_bit_exact(ctx, oracle):
    s = W.hex_pprime(14, peclet=0.0)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_ordering("multicolour")
    x = np.zeros(s.n)
    r = ctx.solve(ocsl.PCG, s.value, s.b, x, tol=1e-10)
    assert r["status"] == 0
    xo, rc, it = oracle_permuted(oracle, oracle.pcg_tol, s, np.zeros(s.n), tol=1e-10)
    assert np.array_equal(x, xo) and r["iterations"] == it


@pytest.mark.parametrize("k", range(4))
def test_multicolour_ir32_reaches_tolerance(ctx, oracle, k):
    s = systems()[k]
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_ordering("multicolour")
    x = np.zeros(s.n)
    r = ctx.solve(ocsl.ILU_BICGSTAB_IR32, s.value, s.b, x, tol=1e-10)
    assert r["status"] == 0 and r["outer_iterations"] >= 1, r
    assert oracle.true_relres(s.row_ptr, s.column_index, s.value, s.b, x) <= 1e-10
    assert r["residual"] <= 1e-10


def test_device_multi_and_natural_switch(ctx, oracle, torch_cuda):
    torch = torch_cuda
    s = W.hex_pprime(10, 9, 8)
    ctx.set_pattern(s.row_ptr, s.column_index)
    x_nat = np.zeros(s.n)
    ctx.solve(ocsl.ILU_BICGSTAB, s.value, s.b, x_nat)
    ctx.set_ordering("multicolour")
    A = torch.from_numpy(s.value).cuda()
    B = torch.stack([torch.from_numpy(s.b), torch.from_numpy(2.0 * s.b)]).cuda()
    X = torch.zeros_like(B)
    res = ctx.solve_multi_device(ocsl.ILU_BICGSTAB_IR32, A, B, X)
    assert all(r["status"] == 0 for r in res)
    for q in range(2):
        xq = X[q].cpu().numpy()
        assert oracle.true_relres(s.row_ptr, s.column_index, s.value, B[q].cpu().numpy(),
                                  xq) <= 1e-10
    Xd = torch.zeros(s.n, dtype=torch.float64, device="cuda")
    r = ctx.solve_device(ocsl.ILU_BICGSTAB, A, B[0].contiguous(), Xd)
    xo, _, it = oracle_permuted(oracle, oracle.bicgstab_tol, s, np.zeros(s.n))
    assert r["status"] == 0 and np.array_equal(Xd.cpu().numpy(), xo) and r["iterations"] == it
    # the reference-faithful methods ignore the ordering
    x = np.zeros(s.n)
    ctx.solve(ocsl.BICGSTAB_REF, s.value, s.b, x)
    xr, _, _ = oracle.bicgstab_ref(s.row_ptr, s.column_index, s.value, s.b, np.zeros(s.n))
    assert np.array_equal(x, xr)
    ctx.set_ordering("natural")
    x = np.zeros(s.n)
    ctx.solve(ocsl.ILU_BICGSTAB, s.value, s.b, x)
    assert np.array_equal(x, x_nat)


def test_multicolour_profile_and_pattern_change(ctx):
    s = W.hex_pprime(8)
    ctx.set_pattern(s.row_ptr, s.column_index)
    ctx.set_ordering("multicolour")
    ctx.profile(True)
    x = np.zeros(s.n)
    assert ctx.solve(ocsl.ILU_BICGSTAB, s.value, s.b, x)["status"] == 0
    prof = ctx.profile_read()
    ctx.profile(False)
    assert prof["fw_sweep_f64"][1] > 0 and prof["spmv_f64"][1] > 0
    # a new pattern drops the permuted one; the next solve builds it again
    t = W.tet_pprime(3)
    ctx.set_pattern(t.row_ptr, t.column_index)
    assert ctx.ordering_info()["colours"] == 0
    x = np.zeros(t.n)
    assert ctx.solve(ocsl.ILU_BICGSTAB, t.value, t.b, x)["status"] == 0
    assert ctx.ordering_info()["colours"] > 2


@pytest.mark.parametrize("k", range(3))
def test_range_sweeps_on_permuted_pattern_bit_exact(ctx, oracle, torch_cuda, k):
    """A multicolour-ordered pattern handed to ocsl_set_pattern directly: its
    level schedule is a few contiguous row ranges, swept one launch per
    level (sweep kind 5); forward and backward sweeps equal the oracle's."""
    torch = torch_cuda
    s = systems()[k]
    perm, colours = OC.colour_order(s.row_ptr, s.column_index)
    rp, col, val, b = OC.permuted_system(s, perm)
    ctx.set_pattern(rp, col)
    if k < 2:  # red-black: two levels each way
        assert ctx.sweep_info()["kind"] == 5
    Mh = oracle.ilu(rp, col, val)
    M = torch.from_numpy(Mh).cuda()
    B = torch.from_numpy(b).cuda()
    Y, X = torch.empty_like(B), torch.empty_like(B)
    ctx.forsub_device(M, B, Y)
    y = oracle.forsub(rp, col, Mh, b)
    assert np.array_equal(Y.cpu().numpy(), y)
    ctx.backsub_device(M, Y, X)
    assert np.array_equal(X.cpu().numpy(), oracle.backsub(rp, col, Mh, y))
